// Host-direct data movement: the GPU reads the caller's FDPS records and id
// lists where they lie in host memory, and writes the results straight into
// the caller's ForceSoft records.
//
// On GB300 the Grace host memory is coherent with the GPU over NVLink-C2C and
// the GPU translates host virtual addresses through the host page tables
// (cudaDevAttrPageableMemoryAccess), so a kernel can load from and store to
// ordinary malloc'd memory at copy-engine speed (about 200 GB/s read and
// 170 GB/s write measured on this part).  These kernels replace the host-side
// packing into pinned staging, the staging copies and the host-side unpacking
// of the reference functors' host code (src/force_gpu_cuda.cu:577-619 send,
// 621-699 dispatch, 831-880 retrieve) with one gather kernel per phase.
//
// The arithmetic is the host packing's, term for term, with every FP64
// operation explicitly rounded (no contraction into FMAs), so both paths give
// bit-identical device arrays.
#include "petar_gpuforce.h"
#include "pgf_internal.cuh"

namespace pgf {
namespace {

__device__ __forceinline__ const double* dptr(const char* base, size_t off) {
    return reinterpret_cast<const double*>(base + off);
}

// ChangeOver members of src/changeover.hpp:64-75 in FP64, rounded to FP32 (as
// make_co in the host packing).
__device__ __forceinline__ CoRec make_co_dev(double r_in, double r_out, double mass, int64_t id) {
    CoRec c;
    const double d = __dsub_rn(r_out, r_in);
    const double norm = __ddiv_rn(1.0, d);
    const double coff = __ddiv_rn(d, __dadd_rn(r_out, r_in));
    c.r_in = __double2float_rn(r_in);
    c.r_out = __double2float_rn(r_out);
    c.norm = __double2float_rn(norm);
    c.coff = __double2float_rn(coff);
    c.pot_off = __double2float_rn(__ddiv_rn(__dadd_rn(1.0, coff), r_out));
    c.mass = __double2float_rn(mass);
    c.id = id;
    return c;
}

__global__ __launch_bounds__(256) void gather_j_kernel(HdSendArgs a) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (int64_t j = t0; j < a.n_epj; j += stride) {
        const char* r = a.epj + j * (int64_t)a.epj_size;
        const double* p = dptr(r, a.epj_off_pos);
        const double x = p[0], y = p[1], z = p[2];
        const double m = *dptr(r, a.epj_off_mass);
        const double rs = *dptr(r, a.epj_off_rs);
        EpjMix e;
        e.x = x;
        e.y = y;
        e.z = z;
        e.m = __double2float_rn(m);
        e.rs2 = __double2float_rn(__dmul_rn(rs, rs));
        a.out_epj[j] = e;
        a.out_epj_m64[j] = m;
        a.out_epj_rs64[j] = rs;
        EpjF32 o;
        o.xh = __double2float_rn(x);
        o.yh = __double2float_rn(y);
        o.zh = __double2float_rn(z);
        o.xl = __double2float_rn(__dsub_rn(x, (double)o.xh));
        o.yl = __double2float_rn(__dsub_rn(y, (double)o.yh));
        o.zl = __double2float_rn(__dsub_rn(z, (double)o.zh));
        o.m = e.m;
        o.rs2 = e.rs2;
        a.out_epj32[j] = o;
        if (a.out_epj_acc32) {
            const double* ac = dptr(r, a.gr_epj_off_acc);
            AccF32 g;
            g.xh = __double2float_rn(ac[0]);
            g.yh = __double2float_rn(ac[1]);
            g.zh = __double2float_rn(ac[2]);
            g.xl = __double2float_rn(__dsub_rn(ac[0], (double)g.xh));
            g.yl = __double2float_rn(__dsub_rn(ac[1], (double)g.yh));
            g.zl = __double2float_rn(__dsub_rn(ac[2], (double)g.zh));
            g.pad0 = g.pad1 = 0.f;
            a.out_epj_acc32[j] = g;
        }
        if (a.out_epj_co) {
            const double status = *dptr(r, a.co_epj_off_status), mbk = *dptr(r, a.co_epj_off_mass_backup);
            // Mass of the pair potential of a neighbour (src/hard.hpp:1458-1476):
            // singles their mass, members their backup mass, others none.
            const double m_pot = (status == 0.0 && mbk == 0.0) ? m : (status < 0.0 ? mbk : 0.0);
            int64_t id;
            memcpy(&id, r + a.co_epj_off_id, sizeof(id));
            a.out_epj_co[j] = make_co_dev(*dptr(r, a.co_epj_off_r_in), *dptr(r, a.co_epj_off_r_out), m_pot, id);
        }
    }
    for (int64_t j = t0; j < a.n_spj; j += stride) {
        const char* r = a.spj + j * (int64_t)a.spj_size;
        const double* p = dptr(r, a.spj_off_pos);
        const double m = *dptr(r, a.spj_off_mass);
        double q[6] = {0, 0, 0, 0, 0, 0};
        if (a.spj_has_quad) {
            const double* qq = dptr(r, a.spj_off_quad);
            for (int k = 0; k < 6; ++k) q[k] = qq[k];
        }
        const double tr = __dadd_rn(__dadd_rn(q[0], q[1]), q[2]);
        SpjMix s;
        s.x = p[0];
        s.y = p[1];
        s.z = p[2];
        s.m = __double2float_rn(m);
        s.pad0 = 0.f;
        s.Q[0] = __double2float_rn(__dsub_rn(__dmul_rn(3.0, q[0]), tr));
        s.Q[1] = __double2float_rn(__dsub_rn(__dmul_rn(3.0, q[1]), tr));
        s.Q[2] = __double2float_rn(__dsub_rn(__dmul_rn(3.0, q[2]), tr));
        s.Q[3] = __double2float_rn(__dmul_rn(3.0, q[3]));
        s.Q[4] = __double2float_rn(__dmul_rn(3.0, q[4]));
        s.Q[5] = __double2float_rn(__dmul_rn(3.0, q[5]));
        s.tr = __double2float_rn(tr);
        s.pad1 = 0.f;
        a.out_spj[j] = s;
        SpjQ64 d;
        d.m = m;
        for (int k = 0; k < 6; ++k) d.q[k] = q[k];
        d.pad = 0.0;
        a.out_spj_q64[j] = d;
        SpjF32 o;
        o.xh = __double2float_rn(s.x);
        o.yh = __double2float_rn(s.y);
        o.zh = __double2float_rn(s.z);
        o.xl = __double2float_rn(__dsub_rn(s.x, (double)o.xh));
        o.yl = __double2float_rn(__dsub_rn(s.y, (double)o.yh));
        o.zl = __double2float_rn(__dsub_rn(s.z, (double)o.zh));
        o.m = s.m;
        o.tr = s.tr;
        for (int c = 0; c < 6; ++c) o.Q[c] = s.Q[c];
        o.pad[0] = o.pad[1] = 0.f;
        a.out_spj32[j] = o;
    }
}

// kIdParts CTAs per walk (grid-stride over the units): each copies a slice
// of the walk's id lists and checks it against the sent arrays; the first
// also writes the walk's EPI rows (with the copies that the parts of a split
// walk read), its box and descriptor(s) and its split record.  Host memory
// answers in
// microseconds and serves whole lines best, so a CTA reads a walk's EPI
// records as contiguous 8-byte words into shared memory (up to kEpiWords per
// round) and its id lists as contiguous 4-byte words, and each thread issues
// all its loads of a round before its first store.  The host sends only
// 8-byte aligned records whose size and offsets are multiples of 8, at most
// 4 KB each.  The CTAs also copy the work-queue order from the pinned host
// table, and the last CTA to finish publishes the id check's outcome.
constexpr int kGatherThreads = 256;
constexpr int kIdBatch = 8;
constexpr int kIdParts = 4;  // CTAs per walk for the id lists
constexpr int kEpiWords = 3072;
constexpr int kEpiPerThread = kEpiWords / kGatherThreads;

__device__ __forceinline__ void write_rows(const HdWalkArgs& a, const WalkSrc& w, int i, const EpiDev& e,
                                           const Accp& ac, const CoRec& co) {
    for (int j = 0; j < w.parts; ++j) {
        const int64_t row = j == 0 ? w.i_off + i : w.rows1 + (int64_t)(j - 1) * w.n_i + i;
        a.out_epi[row] = e;
        if (a.out_epi_acc) a.out_epi_acc[row] = ac;
        if (a.out_epi_co) a.out_epi_co[row] = co;
    }
}

// Loads the 8-byte words [0, n) of src, kEpiPerThread per thread.
__device__ __forceinline__ void load_words(const uint64_t* src, int n, uint64_t (&v)[kEpiPerThread]) {
#pragma unroll
    for (int u = 0; u < kEpiPerThread; ++u) {
        const int q = u * kGatherThreads + (int)threadIdx.x;
        v[u] = q < n ? src[q] : 0ull;
    }
}

__global__ __launch_bounds__(kGatherThreads) void gather_walks_kernel(HdWalkArgs a) {
    __shared__ double red[7][kGatherThreads];
    __shared__ uint64_t ebuf[kEpiWords];
    __shared__ uint64_t wsrc[sizeof(WalkSrc) / 8];
    __shared__ unsigned bad;
    static_assert(sizeof(WalkSrc) % 8 == 0 && sizeof(WalkSrc) / 8 <= kGatherThreads, "walk table entry");
    const int t = threadIdx.x;
    for (int q = blockIdx.x * kGatherThreads + t; q < a.n_desc; q += gridDim.x * kGatherThreads)
        a.order_dst[q] = a.order_src[q];
    const int per_round = a.epi_size ? (int)((size_t)kEpiWords * 8 / a.epi_size) : 1;
    // Unit c = (walk c / kIdParts, slice c % kIdParts of its id lists); the
    // slice-0 unit also does the walk's EPI rows and descriptors.
    const int64_t n_units = (int64_t)a.n_walk * kIdParts;
    for (int64_t c = blockIdx.x; c < n_units; c += gridDim.x) {
        const int k = (int)(c / kIdParts), part = (int)(c - (int64_t)k * kIdParts);
        if (t < (int)(sizeof(WalkSrc) / 8)) wsrc[t] = reinterpret_cast<const uint64_t*>(a.src + k)[t];
        if (t == 0) bad = 0;
        __syncthreads();
        const WalkSrc w = *reinterpret_cast<const WalkSrc*>(wsrc);
        // First round of EPI words in flight while the id lists are copied.
        uint64_t ev[kEpiPerThread];
        const int n0 = part != 0 ? 0 : (w.n_i < per_round ? w.n_i : per_round);
        load_words(reinterpret_cast<const uint64_t*>(w.epi), (int)((size_t)n0 * a.epi_size / 8), ev);
        unsigned b = 0;
        const int e0 = (int)((int64_t)w.n_epj * part / kIdParts), e1 = (int)((int64_t)w.n_epj * (part + 1) / kIdParts);
        const int s0 = (int)((int64_t)w.n_spj * part / kIdParts), s1 = (int)((int64_t)w.n_spj * (part + 1) / kIdParts);
        const int n_id = e1 - e0 > s1 - s0 ? e1 - e0 : s1 - s0;
        for (int q0 = 0; q0 < n_id; q0 += kIdBatch * kGatherThreads) {
            int32_t ve[kIdBatch], vs[kIdBatch];
#pragma unroll
            for (int u = 0; u < kIdBatch; ++u) {
                const int q = q0 + u * kGatherThreads + t;
                ve[u] = e0 + q < e1 ? w.id_epj[e0 + q] : 0;
                vs[u] = s0 + q < s1 ? w.id_spj[s0 + q] : 0;
            }
#pragma unroll
            for (int u = 0; u < kIdBatch; ++u) {
                const int q = q0 + u * kGatherThreads + t;
                if (e0 + q < e1) {
                    b |= (unsigned)ve[u] >= (unsigned)a.n_epj_tot;
                    a.out_id_epj[w.e_off + e0 + q] = ve[u];
                }
                if (s0 + q < s1) {
                    b |= (unsigned)vs[u] >= (unsigned)a.n_spj_tot;
                    a.out_id_spj[w.s_off + s0 + q] = vs[u];
                }
            }
        }
        if (b) atomicOr(&bad, 1u);
        __syncthreads();
        if (t == 0 && bad) {
            atomicOr(a.err, 1);
            atomicMax(a.err + 1, w.walk);
        }
        if (part != 0) {
            __syncthreads();  // wsrc and bad are rewritten by the next unit
            continue;
        }
        double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL}, rs_max = 0.0;
        for (int i0 = 0; i0 < w.n_i; i0 += per_round) {
            const int nr = w.n_i - i0 < per_round ? w.n_i - i0 : per_round;
            const int nw = (int)((size_t)nr * a.epi_size / 8);
            if (i0 > 0) {
                __syncthreads();  // the previous round's records are parsed
                load_words(reinterpret_cast<const uint64_t*>(w.epi + (size_t)i0 * a.epi_size), nw, ev);
            }
#pragma unroll
            for (int u = 0; u < kEpiPerThread; ++u) {
                const int q = u * kGatherThreads + t;
                if (q < nw) ebuf[q] = ev[u];
            }
            __syncthreads();
            for (int i = t; i < nr; i += kGatherThreads) {
                const char* r = reinterpret_cast<const char*>(ebuf) + (size_t)i * a.epi_size;
                const double* p = dptr(r, a.epi_off_pos);
                const EpiDev e{p[0], p[1], p[2], *dptr(r, a.epi_off_rs)};
                Accp ac{0.0, 0.0, 0.0, 0.0};
                if (a.out_epi_acc) {
                    const double* q = dptr(r, a.gr_epi_off_acc);
                    ac = Accp{q[0], q[1], q[2], 0.0};
                }
                CoRec co{};
                if (a.out_epi_co) {
                    int64_t id;
                    memcpy(&id, r + a.co_epi_off_id, sizeof(id));
                    co = make_co_dev(*dptr(r, a.co_epi_off_r_in), *dptr(r, a.co_epi_off_r_out),
                                     *dptr(r, a.co_epi_off_self_mass), id);
                }
                write_rows(a, w, i0 + i, e, ac, co);
                rs_max = fmax(rs_max, e.rs);
                lo[0] = fmin(lo[0], e.x);
                lo[1] = fmin(lo[1], e.y);
                lo[2] = fmin(lo[2], e.z);
                hi[0] = fmax(hi[0], e.x);
                hi[1] = fmax(hi[1], e.y);
                hi[2] = fmax(hi[2], e.z);
            }
        }
        for (int d = 0; d < 3; ++d) {
            red[d][t] = lo[d];
            red[3 + d][t] = hi[d];
        }
        red[6][t] = rs_max;
        __syncthreads();
        for (int s = kGatherThreads / 2; s > 0; s >>= 1) {
            if (t < s) {
                for (int d = 0; d < 3; ++d) {
                    red[d][t] = fmin(red[d][t], red[d][t + s]);
                    red[3 + d][t] = fmax(red[3 + d][t], red[3 + d][t + s]);
                }
                red[6][t] = fmax(red[6][t], red[6][t + s]);
            }
            __syncthreads();
        }
        if (t == 0) {
            WalkDesc d;
            d.epj_begin = w.e_off;
            d.spj_begin = w.s_off;
            d.i_begin = (int32_t)w.i_off;
            d.n_i = w.n_i;
            d.n_epj = w.n_epj;
            d.n_spj = w.n_spj;
            if (w.n_i > 0) {
                // As the host packing: centre of the EPI box, half-extents and
                // the largest r_search rounded up (conservative classification).
                d.cx = __dmul_rn(0.5, __dadd_rn(red[0][0], red[3][0]));
                d.cy = __dmul_rn(0.5, __dadd_rn(red[1][0], red[4][0]));
                d.cz = __dmul_rn(0.5, __dadd_rn(red[2][0], red[5][0]));
                d.hx = __double2float_ru(fmax(__dsub_rn(red[3][0], d.cx), __dsub_rn(d.cx, red[0][0])));
                d.hy = __double2float_ru(fmax(__dsub_rn(red[4][0], d.cy), __dsub_rn(d.cy, red[1][0])));
                d.hz = __double2float_ru(fmax(__dsub_rn(red[5][0], d.cz), __dsub_rn(d.cz, red[2][0])));
                d.rs_max = __double2float_ru(red[6][0]);
            } else {
                d.cx = d.cy = d.cz = 0.0;
                d.hx = d.hy = d.hz = d.rs_max = 0.f;
            }
            d.part = 0;
            d.pad[0] = d.pad[1] = d.pad[2] = 0.f;
            d.rcut2 = w.rcut2;
            // A split walk: part j takes a slice of both lists; parts >= 1
            // read the copy of the walk's rows at rows1 + (j - 1) n_i.
            for (int j = 0; j < w.parts; ++j) {
                WalkDesc q = d;
                if (w.parts > 1) {
                    const int e0 = (int)((int64_t)w.n_epj * j / w.parts), e1 = (int)((int64_t)w.n_epj * (j + 1) / w.parts);
                    const int s0 = (int)((int64_t)w.n_spj * j / w.parts), s1 = (int)((int64_t)w.n_spj * (j + 1) / w.parts);
                    q.epj_begin = d.epj_begin + e0;
                    q.n_epj = e1 - e0;
                    q.spj_begin = d.spj_begin + s0;
                    q.n_spj = s1 - s0;
                }
                if (j == 0) {
                    a.out_walks[k] = q;
                } else {
                    q.i_begin = (int32_t)(w.rows1 + (int64_t)(j - 1) * w.n_i);
                    q.part = j;
                    a.out_walks[w.desc1 + j - 1] = q;
                }
            }
            if (w.parts > 1) a.out_splits[w.split] = SplitRec{(int32_t)w.i_off, (int32_t)w.rows1, w.n_i, w.parts};
        }
        __syncthreads();
    }
    // The outcome: the last CTA to finish sees every CTA's atomics.
    if (t == 0) {
        __threadfence();
        if (atomicAdd(a.err + 2, 1) == (int)gridDim.x - 1) {
            __threadfence();
            const int32_t f = atomicExch(a.err, 0), wmax = atomicExch(a.err + 1, 0);
            a.err[2] = 0;
            a.err[3] = f;
            a.err_host[0] = f;
            a.err_host[1] = wmax;
        }
    }
}

// Results of each walk into the caller's records: acc and pot (FP64), n_ngb
// (4 or 8 bytes) and the modes' extra fields, overwritten as RetrieveForceCUDA
// does (src/force_gpu_cuda.cu:866-875).
__global__ __launch_bounds__(256) void scatter_results_kernel(HdScatterArgs a) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int q = 0; q < 4; ++q) a.flags_host[q] = a.flags_dev[q];
        a.flags_dev[2] = 0;
        a.flags_dev[3] = 0;
    }
    for (int k = blockIdx.x; k < a.n_walk; k += gridDim.x) {
        const ForceDst f = a.dst[k];
        for (int i = threadIdx.x; i < f.n; i += blockDim.x) {
            char* r = f.base + (int64_t)i * (int64_t)a.size;
            const int64_t row = f.row + i;
            if (!a.counts_only) {
                const Accp v = a.accp[row];
                double* acc = reinterpret_cast<double*>(r + a.off_acc);
                acc[0] = v.x;
                acc[1] = v.y;
                acc[2] = v.z;
                *reinterpret_cast<double*>(r + a.off_pot) = v.w;
                if (a.pot_soft) *reinterpret_cast<double*>(r + a.off_pot_soft) = a.pot_soft[row];
                if (a.acorr) {
                    const Accp c = a.acorr[row];
                    double* ac = reinterpret_cast<double*>(r + a.off_acorr);
                    ac[0] = c.x;
                    ac[1] = c.y;
                    ac[2] = c.z;
                }
            }
            if (a.nnb_bytes == 8)
                *reinterpret_cast<int64_t*>(r + a.off_nnb) = a.nnb[row];
            else
                *reinterpret_cast<int32_t*>(r + a.off_nnb) = a.nnb[row];
        }
    }
}

int grid_for(int64_t n, int per_block, int num_sms) {
    int64_t g = (n + per_block - 1) / per_block;
    const int64_t cap = (int64_t)num_sms * 8;
    if (g > cap) g = cap;
    return g < 1 ? 1 : (int)g;
}

}  // namespace

cudaError_t launch_gather_j(const HdSendArgs& a, int num_sms, cudaStream_t s) {
    const int64_t n = a.n_epj > a.n_spj ? a.n_epj : a.n_spj;
    if (n <= 0) return cudaSuccess;
    gather_j_kernel<<<grid_for(n, 256, num_sms), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gather_walks(const HdWalkArgs& a, int num_sms, cudaStream_t s) {
    const int64_t units = (int64_t)a.n_walk * kIdParts;
    int grid = units < num_sms * 8 ? (int)units : num_sms * 8;
    if (grid < 1) grid = 1;  // the outcome is published even with no walk
    gather_walks_kernel<<<grid, kGatherThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_scatter_results(const HdScatterArgs& a, int num_sms, cudaStream_t s) {
    int grid = a.n_walk < num_sms * 8 ? a.n_walk : num_sms * 8;
    if (grid < 1) grid = 1;  // the status words move even with no walk
    scatter_results_kernel<<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace pgf
