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

// One CTA per walk (grid-stride over walks): EPI rows, the walk's box and
// descriptor(s), and its id lists, checked against the sent arrays.
constexpr int kGatherThreads = 256;

__global__ __launch_bounds__(kGatherThreads) void gather_walks_kernel(HdWalkArgs a) {
    __shared__ double red[7][kGatherThreads];
    __shared__ unsigned bad;
    const int t = threadIdx.x;
    for (int k = blockIdx.x; k < a.n_walk; k += gridDim.x) {
        const WalkSrc w = a.src[k];
        if (t == 0) bad = 0;
        double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL}, rs_max = 0.0;
        for (int i = t; i < w.n_i; i += kGatherThreads) {
            const char* r = w.epi + (int64_t)i * (int64_t)a.epi_size;
            const double* p = dptr(r, a.epi_off_pos);
            EpiDev e{p[0], p[1], p[2], *dptr(r, a.epi_off_rs)};
            const int64_t row = w.i_off + i;
            a.out_epi[row] = e;
            if (a.out_epi_acc) {
                const double* ac = dptr(r, a.gr_epi_off_acc);
                a.out_epi_acc[row] = Accp{ac[0], ac[1], ac[2], 0.0};
            }
            if (a.out_epi_co) {
                int64_t id;
                memcpy(&id, r + a.co_epi_off_id, sizeof(id));
                a.out_epi_co[row] = make_co_dev(*dptr(r, a.co_epi_off_r_in), *dptr(r, a.co_epi_off_r_out),
                                                *dptr(r, a.co_epi_off_self_mass), id);
            }
            rs_max = fmax(rs_max, e.rs);
            lo[0] = fmin(lo[0], e.x);
            lo[1] = fmin(lo[1], e.y);
            lo[2] = fmin(lo[2], e.z);
            hi[0] = fmax(hi[0], e.x);
            hi[1] = fmax(hi[1], e.y);
            hi[2] = fmax(hi[2], e.z);
        }
        unsigned b = 0;
        for (int q = t; q < w.n_epj; q += kGatherThreads) {
            const int32_t v = w.id_epj[q];
            b |= (unsigned)v >= (unsigned)a.n_epj_tot;
            a.out_id_epj[w.e_off + q] = v;
        }
        for (int q = t; q < w.n_spj; q += kGatherThreads) {
            const int32_t v = w.id_spj[q];
            b |= (unsigned)v >= (unsigned)a.n_spj_tot;
            a.out_id_spj[w.s_off + q] = v;
        }
        for (int d = 0; d < 3; ++d) {
            red[d][t] = lo[d];
            red[3 + d][t] = hi[d];
        }
        red[6][t] = rs_max;
        __syncthreads();
        if (b) atomicOr(&bad, 1u);
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
            if (bad) {
                atomicOr(a.err, 1);
                atomicMax(a.err + 1, w.walk);
            }
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
        }
        __syncthreads();
    }
}

// Results of each walk into the caller's records: acc and pot (FP64), n_ngb
// (4 or 8 bytes) and the modes' extra fields, overwritten as RetrieveForceCUDA
// does (src/force_gpu_cuda.cu:866-875).
__global__ __launch_bounds__(256) void scatter_results_kernel(HdScatterArgs a) {
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
    if (a.n_walk <= 0) return cudaSuccess;
    const int grid = a.n_walk < num_sms * 8 ? a.n_walk : num_sms * 8;
    gather_walks_kernel<<<grid, kGatherThreads, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_scatter_results(const HdScatterArgs& a, int num_sms, cudaStream_t s) {
    if (a.n_walk <= 0) return cudaSuccess;
    const int grid = a.n_walk < num_sms * 8 ? a.n_walk : num_sms * 8;
    scatter_results_kernel<<<grid, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace pgf
