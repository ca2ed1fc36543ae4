// Mixed-precision soft-force kernel for sm_103a.
//
// Per pair this evaluates the same quantities as the reference GPU kernel
// (src/force_gpu_cuda.cu:50-77 EP-EP with linear cutoff and neighbour count,
// :276-323 EP-SP quadrupole) but arranged for GB300:
//
// * Precision.  Each walk's centre c (centre of its EPI box) is FP64.  j tiles
//   are gathered through the id lists from the FP64 EPJ/SPJ arrays (resident
//   in L2), and x - c is formed in FP64 and rounded to FP32 as the tile is
//   written to shared memory; i-particles get the same treatment once per
//   walk and stay in registers (2 per lane).  Pair arithmetic is FP32 FMA plus
//   rsqrt.approx; each warp's partial sums over one j tile are FP32 and are
//   added into FP64 accumulators at the end of the tile.
// * Exact neighbour counts.  The FP32 test r2 < max(rs_i, rs_j)^2 is done on
//   the float bit patterns with a per-i guard band of K ulps that bounds the
//   FP32 error of r2 (see kband below).  Pairs below rs2 - K ulps are counted,
//   pairs above rs2 + K ulps are not, and a (lane, tile-slice) holding any pair
//   inside the band is not counted here: it is pushed as a Retest record and
//   recounted in FP64 by retest_kernel with the oracle's exact expression.
// * Work distribution.  A persistent grid takes walks from a queue sorted by
//   descending n_i * (n_epj + n_spj).  A 256-thread block holds up to 512
//   i-particles (8 warps x 32 lanes x 2); walks with fewer i split each j tile
//   between warps (n_jslice = 8 / n_ichunk) and reduce the slices through
//   shared memory in FP64.
// * EP-SP uses the traceless form Q = 3q - tr(q) I of the raw quadrupole
//   (algebraically the reference's formula, with eps2 kept through
//   c = -tr(q) eps2): pot = -G (m/r + (d.Q.d + c)/(2 r^5)),
//   acc = G ((m/r^3 + 2.5 (d.Q.d + c)/r^7) d - Q.d/r^5), d = xj - xi.
#include "pgf_internal.cuh"

namespace pgf {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kIPerLane = 2;
constexpr int kIPerWarp = 32 * kIPerLane;
constexpr int kIPerPass = kWarps * kIPerWarp;  // 512 i-particles per pass
constexpr int kTileEP = 256;
constexpr int kTileSP = 128;
constexpr int kKMax = 1 << 22;

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Guard band (in float ulps of rs2) for the FP32 neighbour test of one
// i-particle.  With u = 2^-24, D = max_c |xi - c|_c, and walk-relative
// coordinates rounded once from FP64, each FP32 difference d_c satisfies
// |d_c - (xj - xi)_c| <= 2.0000002 u (|d_c| + D); the FP32 r2 (three FMAs)
// then differs from the exact r2 + eps2 by at most (7 u + 6.93 u D / r) r2 near
// the threshold, where r >= r_ref = sqrt(rs_i^2 - eps2); rounding rs2 to
// float adds u rs2.  One ulp of a float x is at least u x, so the bound is
// below 8 + 6.93 D / r_ref ulps; K doubles it and adds 16.
__device__ __forceinline__ int kband(double D, double rs, double eps2) {
    const double r2ref = rs * rs - eps2;
    if (!(r2ref > 0.0)) return kKMax;
    const double k = 32.0 + 16.0 * D / sqrt(r2ref);
    return k >= double(kKMax) ? kKMax : int(k) + 1;
}

struct __align__(16) Smem {
    float4 ep[kTileEP];
    float rs2[kTileEP];
    float4 sp[kTileSP][3];
    double red[kIPerPass][4];
    int redn[kIPerPass];
    int w;
};

// Exact FP64 count of the pairs (i, id_epj[j_begin .. j_begin + n)).
__device__ int exact_count(const Params& p, int gi, int64_t j_begin, int n) {
    const EpiDev ei = p.epi[gi];
    int c = 0;
    for (int k = 0; k < n; ++k) {
        const int id = p.id_epj[j_begin + k];
        const EpjDev e = p.epj[id];
        c += exact_neighbour(ei.x, ei.y, ei.z, ei.rs, e.x, e.y, e.z, p.epj_rs[id], p.eps2);
    }
    return c;
}

__global__ __launch_bounds__(kThreads, 2) void mixed_kernel(Params p) {
    __shared__ Smem s;
    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const double eps2d = p.eps2;
    const float eps2 = (float)p.eps2;

    for (;;) {
        if (tid == 0) s.w = atomicAdd(p.queue_head, 1);
        __syncthreads();
        const int wq = s.w;
        __syncthreads();
        if (wq >= p.n_walk) break;
        const WalkDesc wd = p.walks[p.order[wq]];
        const double cx = wd.cx, cy = wd.cy, cz = wd.cz;
        const float rcut2 = (float)wd.rcut2;

        for (int ipass = 0; ipass < wd.n_i; ipass += kIPerPass) {
            const int nip = min(kIPerPass, wd.n_i - ipass);
            const int n_ichunk = (nip + kIPerWarp - 1) / kIPerWarp;
            const int n_js = kWarps / n_ichunk;
            const int ichunk = warp % n_ichunk;
            const int js = warp / n_ichunk;
            const bool active = js < n_js;

            float xi[kIPerLane], yi[kIPerLane], zi[kIPerLane], rsi2[kIPerLane];
            int kb[kIPerLane], gi[kIPerLane];
            bool valid[kIPerLane];
            double acc[kIPerLane][4];
            int cnt[kIPerLane];
#pragma unroll
            for (int k = 0; k < kIPerLane; ++k) {
                const int li = ichunk * kIPerWarp + k * 32 + lane;
                valid[k] = active && li < nip;
                gi[k] = wd.i_begin + ipass + li;
                xi[k] = yi[k] = zi[k] = 0.f;
                rsi2[k] = 0.f;
                kb[k] = 0;
                if (valid[k]) {
                    const EpiDev e = p.epi[gi[k]];
                    const double dx = e.x - cx, dy = e.y - cy, dz = e.z - cz;
                    xi[k] = (float)dx;
                    yi[k] = (float)dy;
                    zi[k] = (float)dz;
                    rsi2[k] = (float)(e.rs * e.rs);
                    const double D = fmax(fabs(dx), fmax(fabs(dy), fabs(dz)));
                    kb[k] = kband(D, e.rs, eps2d);
                }
                acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.0;
                cnt[k] = 0;
            }

            // ---- EP-EP: linear cutoff + neighbour count ----
            for (int t0 = 0; t0 < wd.n_epj; t0 += kTileEP) {
                const int nt = min(kTileEP, wd.n_epj - t0);
                __syncthreads();
                for (int jj = tid; jj < nt; jj += kThreads) {
                    const int id = p.id_epj[wd.epj_begin + t0 + jj];
                    const EpjDev e = p.epj[id];
                    s.ep[jj] = make_float4((float)(e.x - cx), (float)(e.y - cy), (float)(e.z - cz), (float)e.m);
                    s.rs2[jj] = p.epj_rs2f[id];
                }
                __syncthreads();
                if (active) {
                    const int per = (nt + n_js - 1) / n_js;
                    const int j0 = min(nt, js * per);
                    const int j1 = min(nt, j0 + per);
                    float a[kIPerLane][4];
                    int c[kIPerLane];
                    bool amb[kIPerLane];
#pragma unroll
                    for (int k = 0; k < kIPerLane; ++k) {
                        a[k][0] = a[k][1] = a[k][2] = a[k][3] = 0.f;
                        c[k] = 0;
                        amb[k] = false;
                    }
#pragma unroll 4
                    for (int j = j0; j < j1; ++j) {
                        const float4 q = s.ep[j];
                        const float rsj2 = s.rs2[j];
#pragma unroll
                        for (int k = 0; k < kIPerLane; ++k) {
                            const float dx = q.x - xi[k];
                            const float dy = q.y - yi[k];
                            const float dz = q.z - zi[k];
                            float r2 = fmaf(dx, dx, eps2);
                            r2 = fmaf(dy, dy, r2);
                            r2 = fmaf(dz, dz, r2);
                            const float rs2 = fmaxf(rsi2[k], rsj2);
                            const int e = __float_as_int(r2) - __float_as_int(rs2) + kb[k];
                            c[k] += (int)((unsigned)e >> 31);
                            amb[k] |= (unsigned)e < (unsigned)(2 * kb[k]);
                            const float ri = rsqrt_approx(fmaxf(r2, rcut2));
                            const float mri = q.w * ri;
                            const float mri3 = mri * (ri * ri);
                            a[k][0] = fmaf(mri3, dx, a[k][0]);
                            a[k][1] = fmaf(mri3, dy, a[k][1]);
                            a[k][2] = fmaf(mri3, dz, a[k][2]);
                            a[k][3] -= mri;
                        }
                    }
#pragma unroll
                    for (int k = 0; k < kIPerLane; ++k) {
                        if (!valid[k]) continue;
                        acc[k][0] += (double)a[k][0];
                        acc[k][1] += (double)a[k][1];
                        acc[k][2] += (double)a[k][2];
                        acc[k][3] += (double)a[k][3];
                        if (!amb[k]) {
                            cnt[k] += c[k];
                        } else if (j1 > j0) {
                            const int64_t jb = wd.epj_begin + t0 + j0;
                            const int slot = atomicAdd(p.n_retest, 1);
                            if (slot < p.retest_cap) {
                                Retest r;
                                r.j_begin = jb;
                                r.i = gi[k];
                                r.n = j1 - j0;
                                p.retest[slot] = r;
                            } else {
                                cnt[k] += exact_count(p, gi[k], jb, j1 - j0);
                            }
                        }
                    }
                }
            }

            // ---- EP-SP: quadrupole, no cutoff ----
            for (int t0 = 0; t0 < wd.n_spj; t0 += kTileSP) {
                const int nt = min(kTileSP, wd.n_spj - t0);
                __syncthreads();
                for (int jj = tid; jj < nt; jj += kThreads) {
                    const int id = p.id_spj[wd.spj_begin + t0 + jj];
                    const SpjDev e = p.spj[id];
                    const float qxx = (float)e.q[0], qyy = (float)e.q[1], qzz = (float)e.q[2];
                    const float tr = qxx + qyy + qzz;
                    s.sp[jj][0] = make_float4((float)(e.x - cx), (float)(e.y - cy), (float)(e.z - cz), (float)e.m);
                    s.sp[jj][1] = make_float4(3.f * qxx - tr, 3.f * qyy - tr, 3.f * qzz - tr, 3.f * (float)e.q[3]);
                    s.sp[jj][2] = make_float4(3.f * (float)e.q[4], 3.f * (float)e.q[5], -tr * eps2, 0.f);
                }
                __syncthreads();
                if (active) {
                    const int per = (nt + n_js - 1) / n_js;
                    const int j0 = min(nt, js * per);
                    const int j1 = min(nt, j0 + per);
                    float a[kIPerLane][4];
#pragma unroll
                    for (int k = 0; k < kIPerLane; ++k) a[k][0] = a[k][1] = a[k][2] = a[k][3] = 0.f;
#pragma unroll 2
                    for (int j = j0; j < j1; ++j) {
                        const float4 q0 = s.sp[j][0];
                        const float4 q1 = s.sp[j][1];
                        const float4 q2 = s.sp[j][2];
#pragma unroll
                        for (int k = 0; k < kIPerLane; ++k) {
                            const float dx = q0.x - xi[k];
                            const float dy = q0.y - yi[k];
                            const float dz = q0.z - zi[k];
                            float r2 = fmaf(dx, dx, eps2);
                            r2 = fmaf(dy, dy, r2);
                            r2 = fmaf(dz, dz, r2);
                            const float ri = rsqrt_approx(r2);
                            // Q.d with Q = (xx yy zz xy | xz yz)
                            const float qdx = fmaf(q1.x, dx, fmaf(q1.w, dy, q2.x * dz));
                            const float qdy = fmaf(q1.w, dx, fmaf(q1.y, dy, q2.y * dz));
                            const float qdz = fmaf(q2.x, dx, fmaf(q2.y, dy, q1.z * dz));
                            const float sq = fmaf(qdx, dx, fmaf(qdy, dy, fmaf(qdz, dz, q2.z)));
                            const float ri2 = ri * ri;
                            const float ri3 = ri2 * ri;
                            const float ri5 = ri3 * ri2;
                            const float t = sq * ri5;
                            const float A = fmaf(t * ri2, 2.5f, q0.w * ri3);
                            a[k][0] = fmaf(A, dx, fmaf(-ri5, qdx, a[k][0]));
                            a[k][1] = fmaf(A, dy, fmaf(-ri5, qdy, a[k][1]));
                            a[k][2] = fmaf(A, dz, fmaf(-ri5, qdz, a[k][2]));
                            a[k][3] = fmaf(-0.5f, t, fmaf(-q0.w, ri, a[k][3]));
                        }
                    }
#pragma unroll
                    for (int k = 0; k < kIPerLane; ++k) {
                        if (!valid[k]) continue;
                        acc[k][0] += (double)a[k][0];
                        acc[k][1] += (double)a[k][1];
                        acc[k][2] += (double)a[k][2];
                        acc[k][3] += (double)a[k][3];
                    }
                }
            }

            // ---- reduce the j-slices and write ----
            __syncthreads();
            const int stride = n_ichunk * kIPerWarp;
            if (active) {
#pragma unroll
                for (int k = 0; k < kIPerLane; ++k) {
                    const int slot = js * stride + ichunk * kIPerWarp + k * 32 + lane;
                    s.red[slot][0] = acc[k][0];
                    s.red[slot][1] = acc[k][1];
                    s.red[slot][2] = acc[k][2];
                    s.red[slot][3] = acc[k][3];
                    s.redn[slot] = cnt[k];
                }
            }
            __syncthreads();
            if (active && js == 0) {
                const double G = p.G;
#pragma unroll
                for (int k = 0; k < kIPerLane; ++k) {
                    if (!valid[k]) continue;
                    const int base = ichunk * kIPerWarp + k * 32 + lane;
                    double r0 = 0, r1 = 0, r2 = 0, r3 = 0;
                    int n = 0;
                    for (int q = 0; q < n_js; ++q) {
                        const int slot = q * stride + base;
                        r0 += s.red[slot][0];
                        r1 += s.red[slot][1];
                        r2 += s.red[slot][2];
                        r3 += s.red[slot][3];
                        n += s.redn[slot];
                    }
                    p.out_accp[gi[k]] = make_double4(G * r0, G * r1, G * r2, G * r3);
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
    const int n_rec = min(*p.n_retest, p.retest_cap);
    const int lane = threadIdx.x & 31;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int r = gw; r < n_rec; r += nw) {
        const Retest rec = p.retest[r];
        const EpiDev ei = p.epi[rec.i];
        int c = 0;
        for (int k = lane; k < rec.n; k += 32) {
            const int id = p.id_epj[rec.j_begin + k];
            const EpjDev e = p.epj[id];
            c += exact_neighbour(ei.x, ei.y, ei.z, ei.rs, e.x, e.y, e.z, p.epj_rs[id], p.eps2);
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
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mixed_kernel, kThreads, 0);
    if (e != cudaSuccess) return e;
    int grid = num_sms * (per_sm > 0 ? per_sm : 1);
    if (grid > p.n_walk) grid = p.n_walk;
    mixed_kernel<<<grid, kThreads, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_retest(const Params& p, cudaStream_t s, int num_sms) {
    retest_kernel<<<num_sms * 2, 256, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace pgf
