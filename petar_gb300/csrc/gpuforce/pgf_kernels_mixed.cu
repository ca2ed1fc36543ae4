// Mixed-precision soft-force kernel for sm_103a.
//
// Per pair this evaluates the quantities of the reference GPU kernel
// (src/force_gpu_cuda.cu:50-77: EP-EP with linear cutoff and neighbour count;
// :276-323: EP-SP quadrupole), arranged for GB300's FP32 pipe.
//
// Precision
//   Each walk has an FP64 centre c (centre of its EPI box).  i-particles and
//   staged j-particles are turned into walk-relative coordinates x - c in FP64
//   and rounded to FP32 ("hi").  Pair arithmetic is FP32 FMA plus
//   rsqrt.approx.  Per-thread FP32 partial sums are flushed into FP64
//   accumulators (in shared memory) every kFlush pairs.
// Near and far EPJ
//   Every staged EPJ tile is split, with a conservative FP32 test against the
//   walk's EPI box, into
//   * far entries: farther than max(r_search of any i, r_search_j, r_out) from
//     every i (with a 0.1% margin).  For them the neighbour test is false and
//     the cutoff max(r2, r_out^2) is r2 for every i, so the pair reduces to
//     plain gravity (14 FP32 instructions);
//   * near entries (a few percent of pairs): they also carry the FP32 rounding
//     residual x - c - hi ("lo"), so d = (hi_j - hi_i) + (lo_j - lo_i) keeps
//     about 2u relative accuracy even for binary companions 1e-5 apart inside
//     a walk 0.1 wide; these pairs get the cutoff and the neighbour test.
// Exact neighbour counts
//   The FP32 test r2 < max(rs_i, rs_j)^2 is done on float bit patterns with a
//   per-i guard band of K ulps that bounds the FP32 error (kband_near).  Pairs
//   more than K ulps below rs2 are counted, pairs more than K ulps above are
//   not.  If any pair of (i, tile) falls inside the band, every thread drops
//   its count of that (i, tile) and one thread pushes a Retest record: the
//   retest kernel recounts the tile in FP64 with the oracle's expression.
// Work distribution
//   A persistent grid takes walks from a queue sorted by descending cost.  A
//   pass holds up to 512 i-particles, 2 per thread; the S = ceil(n_i / 2)
//   threads of one j-slice cover the pass and floor(256 / S) slices split each
//   j tile, so small walks still keep most threads busy.  Tiles are double
//   buffered: while a tile is computed, each thread already holds the next
//   tile's record (and the id of the one after) in registers.
// EP-SP
//   Traceless Q = 3q - tr(q) I is precomputed in FP64 on the host; with
//   c = -tr(q) eps2 (the reference keeps eps2 inside its r^2):
//   pot = -G (m/r + (d.Q.d + c)/(2 r^5)),
//   acc = G ((m/r^3 + 2.5 (d.Q.d + c)/r^7) d - Q.d/r^5),  d = xj - xi.
#include "pgf_internal.cuh"

namespace pgf {
namespace {

#ifndef PGF_THREADS
#define PGF_THREADS 256
#endif
#ifndef PGF_KI
#define PGF_KI 2
#endif
#ifndef PGF_MINB
#define PGF_MINB 2
#endif
#ifndef PGF_FAR_UNROLL
#define PGF_FAR_UNROLL 4
#endif
#ifndef PGF_NEAR_UNROLL
#define PGF_NEAR_UNROLL 2
#endif
#ifndef PGF_SP_UNROLL
#define PGF_SP_UNROLL 2
#endif

constexpr int kThreads = PGF_THREADS;
constexpr int kWarps = kThreads / 32;
constexpr int kI = PGF_KI;               // i-particles per thread
constexpr int kMaxPass = kThreads * kI;  // i-particles per pass
constexpr int kTileEP = kThreads;        // one EPJ per thread per tile
constexpr int kTileSP = kThreads / 2;    // two threads stage one SPJ
constexpr int kFlush = 256;              // pairs per thread between FP64 flushes
constexpr int kKMax = 1 << 22;
constexpr int kNearUnroll = PGF_NEAR_UNROLL;
constexpr int kFarUnroll = PGF_FAR_UNROLL;
constexpr int kSpUnroll = PGF_SP_UNROLL;

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Guard band, in float ulps of rs2, for the near-pair neighbour test of one
// i-particle at distance D (max norm) from the walk centre.  With u = 2^-24
// and hi/lo walk-relative coordinates, |d_c - (xj - xi)_c| <= 2u |d_c| +
// 2.2e-14 D, so the FP32 r2 (three FMAs) is within (7u + 7.6e-14 D / r) of
// r2 + eps2 near the threshold, r >= r_ref = sqrt(rs_i^2 - eps2); rounding
// rs2 to float adds u.  One ulp of x is at least u x: the bound is below
// 8 + 1.3e-6 D / r_ref ulps.  K is more than twice that.
__device__ __forceinline__ int kband_near(double D, double rs, double eps2) {
    const double r2ref = rs * rs - eps2;
    if (!(r2ref > 0.0)) return kKMax;
    const double k = 48.0 + 1e-5 * D / sqrt(r2ref);
    return k >= double(kKMax) ? kKMax : int(k) + 1;
}

struct Smem {
    float4 nh[2][kTileEP];  // near EPJ: hi x, y, z, m
    float4 nl[2][kTileEP];  // near EPJ: lo x, y, z, rs2
    float4 fr[2][kTileEP];  // far EPJ:  hi x, y, z, m
    float4 sp[2][kTileSP][3];
    double acc[kI][4][kThreads];  // FP64 accumulators, one slot per thread
    int cnt[kI][kThreads];
    unsigned flag[kMaxPass];      // ambiguity mark (tile generation) per i slot
    int wcount[kWarps];           // near entries per warp of the tile being staged
    int w;
};

// Exact FP64 count of the pairs (i, id_epj[j_begin .. j_begin + n)).
__device__ int exact_count(const Params& p, int gi, int64_t j_begin, int n) {
    const EpiDev ei = p.epi[gi];
    int c = 0;
    for (int k = 0; k < n; ++k) {
        const int id = p.id_epj[j_begin + k];
        const EpjMix e = p.epj[id];
        c += exact_neighbour(ei.x, ei.y, ei.z, ei.rs, e.x, e.y, e.z, p.epj_rs64[id], p.eps2);
    }
    return c;
}

struct TileRef {
    bool ep;       // EPJ tile (else SPJ)
    int64_t base;  // first list entry of the tile
    int nt;        // entries in the tile
};

__device__ __forceinline__ TileRef tile_ref(const WalkDesc& wd, int t, int n_ept) {
    TileRef r;
    if (t < n_ept) {
        r.ep = true;
        r.base = wd.epj_begin + (int64_t)t * kTileEP;
        r.nt = min(kTileEP, wd.n_epj - t * kTileEP);
    } else {
        const int u = t - n_ept;
        r.ep = false;
        r.base = wd.spj_begin + (int64_t)u * kTileSP;
        r.nt = min(kTileSP, wd.n_spj - u * kTileSP);
    }
    return r;
}

// Entry of a tile this thread stages: EPJ tiles one per thread, SPJ tiles one
// half record per thread.
__device__ __forceinline__ int entry_of(bool ep, int tid) { return ep ? tid : (tid >> 1); }

__device__ __forceinline__ int load_id(const Params& p, const TileRef& r, int tid) {
    const int e = entry_of(r.ep, tid);
    if (e >= r.nt) return -1;
    return r.ep ? __ldg(p.id_epj + r.base + e) : __ldg(p.id_spj + r.base + e);
}

__device__ __forceinline__ void load_rec(const Params& p, bool ep, int id, int tid, uint4& r0, uint4& r1) {
    if (id < 0) return;
    const uint4* src = ep ? reinterpret_cast<const uint4*>(p.epj + id)
                          : reinterpret_cast<const uint4*>(p.spj + id) + 2 * (tid & 1);
    r0 = __ldg(src);
    r1 = __ldg(src + 1);
}

__device__ __forceinline__ double as_double(unsigned lo, unsigned hi) {
    return __hiloint2double((int)hi, (int)lo);
}

__global__ __launch_bounds__(kThreads, PGF_MINB) void mixed_kernel(Params p) {
    if (p.input_err && *p.input_err) return;  // the inputs failed their check: run nothing
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem& s = *reinterpret_cast<Smem*>(smem_raw);
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const unsigned lane_lt = (1u << lane) - 1u;
    const double eps2d = p.eps2;
    const float eps2 = (float)p.eps2;
    unsigned gen = 0;

    for (int i = tid; i < kMaxPass; i += kThreads) s.flag[i] = 0u;

    const int n_walk = walk_count(p);
    for (;;) {
        __syncthreads();
        if (tid == 0) s.w = atomicAdd(p.queue_head, 1);
        __syncthreads();
        const int wq = s.w;
        if (wq >= n_walk) break;
        const int widx = p.order[wq];
        const WalkDesc wd = p.walks[widx];
        const double cx = wd.cx, cy = wd.cy, cz = wd.cz;
        const float rcut2 = (float)wd.rcut2;
        const float rsmax2 = wd.rs_max * wd.rs_max;
        const float hmax = fmaxf(wd.hx, fmaxf(wd.hy, wd.hz));
        const int n_ept = (wd.n_epj + kTileEP - 1) / kTileEP;
        const int n_t = n_ept + (wd.n_spj + kTileSP - 1) / kTileSP;

        for (int ipass = 0; ipass < wd.n_i; ipass += kMaxPass) {
            const int nip = min(kMaxPass, wd.n_i - ipass);
            const int S = (nip + kI - 1) / kI;
            const int n_js = kThreads / S;
            const int js = tid / S;
            const int slot = tid - js * S;
            const bool active = js < n_js;

            float xih[kI], yih[kI], zih[kI], xil[kI], yil[kI], zil[kI], rsi2[kI];
            int kb[kI], gi[kI], li[kI], cnt[kI];
            bool valid[kI];
            float a[kI][4];
#pragma unroll
            for (int k = 0; k < kI; ++k) {
                li[k] = slot + k * S;
                valid[k] = active && li[k] < nip;
                gi[k] = wd.i_begin + ipass + li[k];
                xih[k] = yih[k] = zih[k] = xil[k] = yil[k] = zil[k] = 0.f;
                rsi2[k] = 0.f;
                kb[k] = 0;
                cnt[k] = 0;
                if (valid[k]) {
                    const EpiDev e = p.epi[gi[k]];
                    const double dx = e.x - cx, dy = e.y - cy, dz = e.z - cz;
                    xih[k] = (float)dx;
                    yih[k] = (float)dy;
                    zih[k] = (float)dz;
                    xil[k] = (float)(dx - (double)xih[k]);
                    yil[k] = (float)(dy - (double)yih[k]);
                    zil[k] = (float)(dz - (double)zih[k]);
                    rsi2[k] = (float)(e.rs * e.rs);
                    kb[k] = kband_near(fmax(fabs(dx), fmax(fabs(dy), fabs(dz))), e.rs, eps2d);
                }
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    a[k][c] = 0.f;
                    s.acc[k][c][tid] = 0.0;
                }
            }
            int since = 0;

            // ---- staging of a tile into a buffer: decode, classify, compact ----
            // Registers carried from the decode to the write phase.
            float sx = 0.f, sy = 0.f, sz = 0.f, sm = 0.f, slx = 0.f, sly = 0.f, slz = 0.f, srs2 = 0.f;
            float4 q1 = make_float4(0.f, 0.f, 0.f, 0.f), q2 = q1;
            unsigned bal_near = 0u, bal_far = 0u;
            bool st_near = false, st_valid = false;
            uint4 r0 = make_uint4(0, 0, 0, 0), r1 = r0;

            auto decode = [&](const TileRef& r) {
                const int e = entry_of(r.ep, tid);
                st_valid = e < r.nt;
                st_near = false;
                if (r.ep) {
                    if (st_valid) {
                        const double dx = as_double(r0.x, r0.y) - cx;
                        const double dy = as_double(r0.z, r0.w) - cy;
                        const double dz = as_double(r1.x, r1.y) - cz;
                        sx = (float)dx;
                        sy = (float)dy;
                        sz = (float)dz;
                        sm = __uint_as_float(r1.z);
                        srs2 = __uint_as_float(r1.w);
                        const float ex = fmaxf(fabsf(sx) - wd.hx, 0.f);
                        const float ey = fmaxf(fabsf(sy) - wd.hy, 0.f);
                        const float ez = fmaxf(fabsf(sz) - wd.hz, 0.f);
                        const float dist2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                        const float R = sqrtf(fmaxf(fmaxf(rsmax2, srs2), rcut2));
                        const float dmax = fmaxf(fabsf(sx), fmaxf(fabsf(sy), fabsf(sz)));
                        const float Rm = R * 1.001f + 1e-6f * (dmax + hmax);
                        st_near = !(dist2 > Rm * Rm);
                        if (st_near) {
                            slx = (float)(dx - (double)sx);
                            sly = (float)(dy - (double)sy);
                            slz = (float)(dz - (double)sz);
                        }
                    }
                    bal_near = __ballot_sync(0xffffffffu, st_valid && st_near);
                    bal_far = __ballot_sync(0xffffffffu, st_valid && !st_near);
                    if (lane == 0) s.wcount[warp] = __popc(bal_near);
                } else if (st_valid) {
                    if ((tid & 1) == 0) {
                        sx = (float)(as_double(r0.x, r0.y) - cx);
                        sy = (float)(as_double(r0.z, r0.w) - cy);
                        sz = (float)(as_double(r1.x, r1.y) - cz);
                        sm = __uint_as_float(r1.z);
                    } else {
                        q1 = make_float4(__uint_as_float(r0.x), __uint_as_float(r0.y), __uint_as_float(r0.z),
                                         __uint_as_float(r0.w));
                        q2 = make_float4(__uint_as_float(r1.x), __uint_as_float(r1.y),
                                         -__uint_as_float(r1.z) * eps2, 0.f);
                    }
                }
            };
            // Writes the decoded entry; returns the near and far counts of the tile.
            auto write = [&](const TileRef& r, int b, int& n_near, int& n_far) {
                const int e = entry_of(r.ep, tid);
                if (r.ep) {
                    int before = 0, total = 0;
#pragma unroll
                    for (int q = 0; q < kWarps; ++q) {
                        const int c = s.wcount[q];
                        before += q < warp ? c : 0;
                        total += c;
                    }
                    if (st_valid) {
                        if (st_near) {
                            const int pos = before + __popc(bal_near & lane_lt);
                            s.nh[b][pos] = make_float4(sx, sy, sz, sm);
                            s.nl[b][pos] = make_float4(slx, sly, slz, srs2);
                        } else {
                            const int pos = min(r.nt, 32 * warp) - before + __popc(bal_far & lane_lt);
                            s.fr[b][pos] = make_float4(sx, sy, sz, sm);
                        }
                    }
                    n_near = total;
                    n_far = r.nt - total;
                } else {
                    if (st_valid) {
                        if ((tid & 1) == 0) {
                            s.sp[b][e][0] = make_float4(sx, sy, sz, sm);
                        } else {
                            s.sp[b][e][1] = q1;
                            s.sp[b][e][2] = q2;
                        }
                    }
                    n_near = r.nt;
                    n_far = 0;
                }
            };

            int nn_cur = 0, nf_cur = 0;
            int id_next = -1;
            if (n_t > 0) {
                const TileRef r = tile_ref(wd, 0, n_ept);
                const int id0 = load_id(p, r, tid);
                load_rec(p, r.ep, id0, tid, r0, r1);
                if (n_t > 1) id_next = load_id(p, tile_ref(wd, 1, n_ept), tid);
                decode(r);
                __syncthreads();
                write(r, 0, nn_cur, nf_cur);
                __syncthreads();
            }

            for (int t = 0; t < n_t; ++t) {
                const int cur = t & 1;
                const TileRef rt = tile_ref(wd, t, n_ept);
                const bool has_next = t + 1 < n_t;
                TileRef rn = rt;
                if (has_next) {
                    rn = tile_ref(wd, t + 1, n_ept);
                    load_rec(p, rn.ep, id_next, tid, r0, r1);
                    id_next = (t + 2 < n_t) ? load_id(p, tile_ref(wd, t + 2, n_ept), tid) : -1;
                }
                int c[kI] = {};
                bool amb[kI] = {};
                if (rt.ep) ++gen;
                if (active) {
                    if (rt.ep) {
                        // near pairs: hi/lo differences, cutoff, neighbour count
                        const int pn = (nn_cur + n_js - 1) / n_js;
                        const int j0 = min(nn_cur, js * pn);
                        const int j1 = min(nn_cur, j0 + pn);
#pragma unroll kNearUnroll
                        for (int j = j0; j < j1; ++j) {
                            const float4 h = s.nh[cur][j];
                            const float4 l = s.nl[cur][j];
#pragma unroll
                            for (int k = 0; k < kI; ++k) {
                                const float dx = (h.x - xih[k]) + (l.x - xil[k]);
                                const float dy = (h.y - yih[k]) + (l.y - yil[k]);
                                const float dz = (h.z - zih[k]) + (l.z - zil[k]);
                                float r2 = fmaf(dx, dx, eps2);
                                r2 = fmaf(dy, dy, r2);
                                r2 = fmaf(dz, dz, r2);
                                const float rs2 = fmaxf(rsi2[k], l.w);
                                const int e = __float_as_int(r2) - __float_as_int(rs2) + kb[k];
                                c[k] += (int)((unsigned)e >> 31);
                                amb[k] |= (unsigned)e < (unsigned)(2 * kb[k]);
                                const float ri = rsqrt_approx(fmaxf(r2, rcut2));
                                const float mri = h.w * ri;
                                const float mri3 = mri * (ri * ri);
                                a[k][0] = fmaf(mri3, dx, a[k][0]);
                                a[k][1] = fmaf(mri3, dy, a[k][1]);
                                a[k][2] = fmaf(mri3, dz, a[k][2]);
                                a[k][3] -= mri;
                            }
                        }
                        // far pairs: plain gravity
                        const int pf = (nf_cur + n_js - 1) / n_js;
                        const int f0 = min(nf_cur, js * pf);
                        const int f1 = min(nf_cur, f0 + pf);
#pragma unroll kFarUnroll
                        for (int j = f0; j < f1; ++j) {
                            const float4 h = s.fr[cur][j];
#pragma unroll
                            for (int k = 0; k < kI; ++k) {
                                const float dx = h.x - xih[k];
                                const float dy = h.y - yih[k];
                                const float dz = h.z - zih[k];
                                float r2 = fmaf(dx, dx, eps2);
                                r2 = fmaf(dy, dy, r2);
                                r2 = fmaf(dz, dz, r2);
                                const float ri = rsqrt_approx(r2);
                                const float mri = h.w * ri;
                                const float mri3 = mri * (ri * ri);
                                a[k][0] = fmaf(mri3, dx, a[k][0]);
                                a[k][1] = fmaf(mri3, dy, a[k][1]);
                                a[k][2] = fmaf(mri3, dz, a[k][2]);
                                a[k][3] -= mri;
                            }
                        }
                        since += (j1 - j0) + (f1 - f0);
#pragma unroll
                        for (int k = 0; k < kI; ++k)
                            if (valid[k] && amb[k]) s.flag[li[k]] = gen;
                    } else {
                        const int ps = (nn_cur + n_js - 1) / n_js;
                        const int j0 = min(nn_cur, js * ps);
                        const int j1 = min(nn_cur, j0 + ps);
#pragma unroll kSpUnroll
                        for (int j = j0; j < j1; ++j) {
                            const float4 q0 = s.sp[cur][j][0];
                            const float4 qa = s.sp[cur][j][1];
                            const float4 qb = s.sp[cur][j][2];
#pragma unroll
                            for (int k = 0; k < kI; ++k) {
                                const float dx = q0.x - xih[k];
                                const float dy = q0.y - yih[k];
                                const float dz = q0.z - zih[k];
                                float r2 = fmaf(dx, dx, eps2);
                                r2 = fmaf(dy, dy, r2);
                                r2 = fmaf(dz, dz, r2);
                                const float ri = rsqrt_approx(r2);
                                // Q.d with (qa | qb) = (xx yy zz xy | xz yz c -)
                                const float qdx = fmaf(qa.x, dx, fmaf(qa.w, dy, qb.x * dz));
                                const float qdy = fmaf(qa.w, dx, fmaf(qa.y, dy, qb.y * dz));
                                const float qdz = fmaf(qb.x, dx, fmaf(qb.y, dy, qa.z * dz));
                                const float sq = fmaf(qdx, dx, fmaf(qdy, dy, fmaf(qdz, dz, qb.z)));
                                const float ri2 = ri * ri;
                                const float ri3 = ri2 * ri;
                                const float ri5 = ri3 * ri2;
                                const float tq = sq * ri5;
                                const float A = fmaf(tq * ri2, 2.5f, q0.w * ri3);
                                a[k][0] = fmaf(A, dx, fmaf(-ri5, qdx, a[k][0]));
                                a[k][1] = fmaf(A, dy, fmaf(-ri5, qdy, a[k][1]));
                                a[k][2] = fmaf(A, dz, fmaf(-ri5, qdz, a[k][2]));
                                a[k][3] = fmaf(-0.5f, tq, fmaf(-q0.w, ri, a[k][3]));
                            }
                        }
                        since += j1 - j0;
                    }
                    if (since >= kFlush) {
#pragma unroll
                        for (int k = 0; k < kI; ++k)
#pragma unroll
                            for (int q = 0; q < 4; ++q) {
                                s.acc[k][q][tid] += (double)a[k][q];
                                a[k][q] = 0.f;
                            }
                        since = 0;
                    }
                }
                if (has_next) decode(rn);
                __syncthreads();  // compute of tile t and the flags are complete
                if (rt.ep && active) {
#pragma unroll
                    for (int k = 0; k < kI; ++k) {
                        if (!valid[k]) continue;
                        if (s.flag[li[k]] != gen) {
                            cnt[k] += c[k];
                        } else if (js == 0) {
                            const int slot_r = atomicAdd(p.n_retest, 1);
                            if (slot_r < p.retest_cap) {
                                Retest rr;
                                rr.j_begin = rt.base;
                                rr.i = gi[k];
                                rr.n = rt.nt;
                                rr.walk = widx;
                                rr.pad = 0;
                                p.retest[slot_r] = rr;
                            } else {
                                cnt[k] += exact_count(p, gi[k], rt.base, rt.nt);
                            }
                        }
                    }
                }
                int nn_next = 0, nf_next = 0;
                if (has_next) write(rn, cur ^ 1, nn_next, nf_next);
                __syncthreads();  // tile t+1 is staged
                nn_cur = nn_next;
                nf_cur = nf_next;
            }

            // ---- reduce the j-slices and write ----
            if (active) {
#pragma unroll
                for (int k = 0; k < kI; ++k) {
#pragma unroll
                    for (int q = 0; q < 4; ++q) s.acc[k][q][tid] += (double)a[k][q];
                    s.cnt[k][tid] = cnt[k];
                }
            }
            __syncthreads();
            if (active && js == 0) {
                const double G = p.G;
#pragma unroll
                for (int k = 0; k < kI; ++k) {
                    if (!valid[k]) continue;
                    double r[4] = {0.0, 0.0, 0.0, 0.0};
                    int n = 0;
                    for (int q = 0; q < n_js; ++q) {
                        const int src = q * S + slot;
#pragma unroll
                        for (int c = 0; c < 4; ++c) r[c] += s.acc[k][c][src];
                        n += s.cnt[k][src];
                    }
                    p.out_accp[gi[k]] = Accp{G * r[0], G * r[1], G * r[2], G * r[3]};
                    p.out_nnb[gi[k]] = n;
                }
            }
            __syncthreads();
        }
    }
}

// One warp per Retest record: exact FP64 recount of its pair range, added to
// the neighbour count the interaction kernel wrote.
__global__ __launch_bounds__(256) void retest_kernel(Params p) {
    if (p.input_err && *p.input_err) return;  // the inputs failed their check: run nothing
    const int n_rec = min(*p.n_retest, p.retest_cap);
    if (p.retest_total && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(p.retest_total, *p.n_retest);
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int r = gw; r < n_rec; r += nw) {
        const Retest rec = p.retest[r];
        const EpiDev ei = p.epi[rec.i];
        int c = 0;
        for (int k = lane; k < rec.n; k += 32) {
            const int id = p.id_epj[rec.j_begin + k];
            const EpjMix e = p.epj[id];
            const int nb = exact_neighbour(ei.x, ei.y, ei.z, ei.rs, e.x, e.y, e.z, p.epj_rs64[id], p.eps2);
            c += nb;
            if (p.epi_co && nb) {
                // Fused changeover mode: the interaction kernel used the linear
                // cutoff for this pair; replace it by the changeover terms.
                const CoRec ci = p.epi_co[rec.i], cj = p.epj_co[id];
                if (ci.id != cj.id) {
                    double d[5];
                    co_pair_diff(ei, ci, e, e.m, cj, p.eps2, p.walks[rec.walk].rcut2, d);
                    atomicAdd(&p.out_accp[rec.i].x, p.G * d[0]);
                    atomicAdd(&p.out_accp[rec.i].y, p.G * d[1]);
                    atomicAdd(&p.out_accp[rec.i].z, p.G * d[2]);
                    atomicAdd(&p.out_accp[rec.i].w, p.G * d[3]);
                    atomicAdd(&p.out_pot_soft[rec.i], p.G * d[4]);
                }
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
        if (lane == 0 && c) atomicAdd(&p.out_nnb[rec.i], c);
    }
}

}  // namespace

cudaError_t launch_mixed(const Params& p, cudaStream_t s, int num_sms) {
    cudaError_t e = cudaMemsetAsync(p.queue_head, 0, sizeof(int32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.n_retest, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return e;
    if (p.n_walk <= 0) return cudaSuccess;
    static int per_sm = 0;
    if (per_sm == 0) {
        e = cudaFuncSetAttribute(mixed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Smem));
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mixed_kernel, kThreads, sizeof(Smem));
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    int grid = num_sms * per_sm;
    if (grid > p.n_walk) grid = p.n_walk;
    mixed_kernel<<<grid, kThreads, sizeof(Smem), s>>>(p);
    return cudaGetLastError();
}

__global__ __launch_bounds__(256) void combine_parts_kernel(const SplitRec* __restrict__ recs, Accp* accp,
                                                            int32_t* nnb, double* pot_soft, Accp* acorr) {
    const SplitRec r = recs[blockIdx.x];
    for (int i = threadIdx.x; i < r.n_i; i += blockDim.x) {
        const int64_t r0 = (int64_t)r.row0 + i;
        Accp a = accp[r0];
        int c = nnb[r0];
        double ps = pot_soft ? pot_soft[r0] : 0.0;
        Accp g = acorr ? acorr[r0] : Accp{0.0, 0.0, 0.0, 0.0};
        for (int k = 1; k < r.n_parts; ++k) {
            const int64_t row = (int64_t)r.rows1 + (int64_t)(k - 1) * r.n_i + i;
            const Accp b = accp[row];
            a.x += b.x;
            a.y += b.y;
            a.z += b.z;
            a.w += b.w;
            c += nnb[row];
            if (pot_soft) ps += pot_soft[row];
            if (acorr) {
                const Accp h = acorr[row];
                g.x += h.x;
                g.y += h.y;
                g.z += h.z;
            }
        }
        accp[r0] = a;
        nnb[r0] = c;
        if (pot_soft) pot_soft[r0] = ps;
        if (acorr) acorr[r0] = g;
    }
}

cudaError_t launch_combine_parts(const SplitRec* recs, int n_recs, Accp* accp, int32_t* nnb, double* pot_soft,
                                 Accp* acorr, cudaStream_t s) {
    if (n_recs <= 0) return cudaSuccess;
    combine_parts_kernel<<<n_recs, 256, 0, s>>>(recs, accp, nnb, pot_soft, acorr);
    return cudaGetLastError();
}

__global__ __launch_bounds__(256) void split_rows_kernel(const SplitRec* __restrict__ recs, EpiDev* epi, CoRec* co,
                                                         Accp* acc) {
    const SplitRec r = recs[blockIdx.x];
    const int64_t total = (int64_t)(r.n_parts - 1) * r.n_i;
    for (int64_t k = threadIdx.x; k < total; k += blockDim.x) {
        const int64_t i = k % r.n_i;
        const int64_t src = (int64_t)r.row0 + i, dst = (int64_t)r.rows1 + k;
        epi[dst] = epi[src];
        if (co) co[dst] = co[src];
        if (acc) acc[dst] = acc[src];
    }
}

cudaError_t launch_split_rows(const SplitRec* recs, int n_recs, EpiDev* epi, CoRec* co, Accp* acc, cudaStream_t s) {
    if (n_recs <= 0) return cudaSuccess;
    split_rows_kernel<<<n_recs, 256, 0, s>>>(recs, epi, co, acc);
    return cudaGetLastError();
}

cudaError_t launch_retest(const Params& p, cudaStream_t s, int num_sms) {
    retest_kernel<<<num_sms * 2, 256, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace pgf
