// KDKDK_4TH gradient-correction pass for sm_103a.
//
// PeTar's fourth-order KDKDK integrator runs a second tree pass per step
// (src/petar.hpp:1123-1140) with CalcCorrectEpEpWithLinearCutoffNoSimd
// (src/soft_force.hpp:89-122) for EPJ and the quadrupole force functor for
// SPJ, accumulated into one cleared ForceSoft per i:
//   acorr = 2 sum_j -m_j / r^3 (da - 3 (dr.da) / r^2 dr)   with dr = x_i - x_j,
//           da = a_i - a_j, r^2 = max(|dr|^2 + eps^2, r_out^2)   (no G)
//   acc   = a_i + G acc_sp,   pot = G pot_sp.
// The reference runs it on the CPU only.
//
// Design: a persistent CTA-synchronous kernel (one pass is as heavy as a force
// evaluation, but it runs once per step).  256 threads pop walks from the
// cost-sorted queue; a pass holds up to 512 i, two per thread, and the
// threads form floor(256 / ceil(n_i / 2)) j-slices.  Threads stage 128-entry
// EPJ tiles (positions as walk-relative (hi, lo) pairs from the FP32 split
// arrays, accelerations as (hi, lo) pairs) and 64-entry SPJ tiles in shared
// memory.  Pair arithmetic is FP32 with both halves, so dr and da are accurate
// to an ulp of themselves for close pairs; partial sums are flushed into
// (hi, lo) FP32 accumulators and the slices are combined in FP64.
#include "pgf_internal.cuh"

namespace pgf {
namespace {

constexpr int kThreadsG = 256;
constexpr int kTileEPG = 128;
constexpr int kTileSPG = 64;
constexpr int kFlushG = 256;

__device__ __forceinline__ float rsqrt_approx_g(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void two_sum_g(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

template <int KU>
struct SmemG {
    float4 ph[kTileEPG];  // EPJ: walk-relative position hi, mass
    float4 pl[kTileEPG];  // EPJ: walk-relative position lo
    float4 ah[kTileEPG];  // EPJ: acceleration hi
    float4 al[kTileEPG];  // EPJ: acceleration lo
    float4 sp[kTileSPG][3];
    float2 acc[KU][7][kThreadsG];  // flushed partials: acorr x, y, z, SP acc x, y, z, SP pot
    int w;
};

__device__ __forceinline__ void flush_into(float2& v, float x) {
    float e;
    two_sum_g(v.x, x, v.x, e);
    v.y += e;
}

// KU i-particles per thread: i = li + k S (k < KU) of a pass of up to
// 256 KU i, with S = ceil(n_i / KU) threads per j-slice; every j read from
// shared memory serves KU pairs.
template <int KU>
__global__ __launch_bounds__(kThreadsG, 2) void gradient_kernel(Params p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemG<KU>& s = *reinterpret_cast<SmemG<KU>*>(smem_raw);
    const int tid = threadIdx.x;
    const float eps2 = (float)p.eps2;
    const int n_walk = walk_count(p);
    for (;;) {
        __syncthreads();
        if (tid == 0) s.w = atomicAdd(p.queue_head, 1);
        __syncthreads();
        const int wq = s.w;
        if (wq >= n_walk) break;
        const WalkDesc wd = p.walks[p.order[wq]];
        const float chx = (float)wd.cx, chy = (float)wd.cy, chz = (float)wd.cz;
        const float clx = (float)(wd.cx - (double)chx), cly = (float)(wd.cy - (double)chy),
                    clz = (float)(wd.cz - (double)chz);
        const float rcut2 = (float)wd.rcut2;
        for (int ipass = 0; ipass < wd.n_i; ipass += kThreadsG * KU) {
            const int nip = min(kThreadsG * KU, wd.n_i - ipass);
            const int S = (nip + KU - 1) / KU;
            const int n_js = kThreadsG / S;
            const int js = tid / S;
            const int li = tid - js * S;
            const bool active = js < n_js;
            float xh[KU], yh[KU], zh[KU], xl[KU], yl[KU], zl[KU];
            float axh[KU], ayh[KU], azh[KU], axl[KU], ayl[KU], azl[KU];
#pragma unroll
            for (int k = 0; k < KU; ++k) {
                xh[k] = yh[k] = zh[k] = xl[k] = yl[k] = zl[k] = 0.f;
                axh[k] = ayh[k] = azh[k] = axl[k] = ayl[k] = azl[k] = 0.f;
                const int ii = li + k * S;
                if (active && ii < nip) {
                    const int gi = wd.i_begin + ipass + ii;
                    const EpiDev e = p.epi[gi];
                    const double dx = e.x - wd.cx, dy = e.y - wd.cy, dz = e.z - wd.cz;
                    xh[k] = (float)dx;
                    yh[k] = (float)dy;
                    zh[k] = (float)dz;
                    xl[k] = (float)(dx - (double)xh[k]);
                    yl[k] = (float)(dy - (double)yh[k]);
                    zl[k] = (float)(dz - (double)zh[k]);
                    const Accp a = p.epi_acc64[gi];
                    axh[k] = (float)a.x;
                    ayh[k] = (float)a.y;
                    azh[k] = (float)a.z;
                    axl[k] = (float)(a.x - (double)axh[k]);
                    ayl[k] = (float)(a.y - (double)ayh[k]);
                    azl[k] = (float)(a.z - (double)azh[k]);
                }
            }
#pragma unroll
            for (int k = 0; k < KU; ++k)
#pragma unroll
                for (int q = 0; q < 7; ++q) s.acc[k][q][tid] = make_float2(0.f, 0.f);
            float g[KU][7];
#pragma unroll
            for (int k = 0; k < KU; ++k)
#pragma unroll
                for (int q = 0; q < 7; ++q) g[k][q] = 0.f;
            int since = 0;
            auto flush = [&]() {
#pragma unroll
                for (int k = 0; k < KU; ++k)
#pragma unroll
                    for (int q = 0; q < 7; ++q) {
                        flush_into(s.acc[k][q][tid], g[k][q]);
                        g[k][q] = 0.f;
                    }
                since = 0;
            };
            // EPJ tiles: the gradient correction of every pair.
            for (int t = 0; t < wd.n_epj; t += kTileEPG) {
                const int nt = min(kTileEPG, wd.n_epj - t);
                __syncthreads();
                if (tid < nt) {
                    const int id = p.id_epj[wd.epj_begin + t + tid];
                    const EpjF32 r = p.epj32[id];
                    const AccF32 a = p.epj_acc32[id];
                    float hx, hy, hz, lx, ly, lz, s_, e_;
                    two_sum_g(r.xh, -chx, s_, e_);
                    two_sum_g(s_, e_ + (r.xl - clx), hx, lx);
                    two_sum_g(r.yh, -chy, s_, e_);
                    two_sum_g(s_, e_ + (r.yl - cly), hy, ly);
                    two_sum_g(r.zh, -chz, s_, e_);
                    two_sum_g(s_, e_ + (r.zl - clz), hz, lz);
                    s.ph[tid] = make_float4(hx, hy, hz, r.m);
                    s.pl[tid] = make_float4(lx, ly, lz, 0.f);
                    s.ah[tid] = make_float4(a.xh, a.yh, a.zh, 0.f);
                    s.al[tid] = make_float4(a.xl, a.yl, a.zl, 0.f);
                }
                __syncthreads();
                if (active) {
                    const int pn = (nt + n_js - 1) / n_js;
                    const int j0 = min(nt, js * pn), j1 = min(nt, j0 + pn);
                    for (int j = j0; j < j1; ++j) {
                        const float4 ph = s.ph[j], pl = s.pl[j], ah = s.ah[j], al = s.al[j];
#pragma unroll
                        for (int k = 0; k < KU; ++k) {
                            // x_j - x_i and a_j - a_i from both halves
                            const float dx = (ph.x - xh[k]) + (pl.x - xl[k]);
                            const float dy = (ph.y - yh[k]) + (pl.y - yl[k]);
                            const float dz = (ph.z - zh[k]) + (pl.z - zl[k]);
                            const float dax = (ah.x - axh[k]) + (al.x - axl[k]);
                            const float day = (ah.y - ayh[k]) + (al.y - ayl[k]);
                            const float daz = (ah.z - azh[k]) + (al.z - azl[k]);
                            float r2 = fmaf(dx, dx, eps2);
                            r2 = fmaf(dy, dy, r2);
                            r2 = fmaf(dz, dz, r2);
                            const float ri = rsqrt_approx_g(fmaxf(r2, rcut2));
                            const float ri2 = ri * ri;
                            const float mr3 = ph.w * ri * ri2;
                            const float drda = fmaf(dx, dax, fmaf(dy, day, dz * daz));
                            const float alpha = 3.f * drda * ri2;
                            // -m/r^3 (da - alpha dr) with dr = -d, da = -(a_j - a_i)
                            g[k][0] = fmaf(mr3, fmaf(-alpha, dx, dax), g[k][0]);
                            g[k][1] = fmaf(mr3, fmaf(-alpha, dy, day), g[k][1]);
                            g[k][2] = fmaf(mr3, fmaf(-alpha, dz, daz), g[k][2]);
                        }
                    }
                    since += j1 - j0;
                    if (since >= kFlushG) flush();
                }
            }
            // SPJ tiles: the quadrupole force (traceless Q, c = -tr(q) eps^2).
            for (int t = 0; t < wd.n_spj; t += kTileSPG) {
                const int nt = min(kTileSPG, wd.n_spj - t);
                __syncthreads();
                if (tid < nt) {
                    const int id = p.id_spj[wd.spj_begin + t + tid];
                    const SpjF32 r = p.spj32[id];
                    const float hx = (r.xh - chx) + (r.xl - clx);
                    const float hy = (r.yh - chy) + (r.yl - cly);
                    const float hz = (r.zh - chz) + (r.zl - clz);
                    s.sp[tid][0] = make_float4(hx, hy, hz, r.m);
                    s.sp[tid][1] = make_float4(r.Q[0], r.Q[1], r.Q[2], r.Q[3]);
                    s.sp[tid][2] = make_float4(r.Q[4], r.Q[5], -r.tr * eps2, 0.f);
                }
                __syncthreads();
                if (active) {
                    const int ps = (nt + n_js - 1) / n_js;
                    const int j0 = min(nt, js * ps), j1 = min(nt, j0 + ps);
                    for (int j = j0; j < j1; ++j) {
                        const float4 q0 = s.sp[j][0], qa = s.sp[j][1], qb = s.sp[j][2];
#pragma unroll
                        for (int k = 0; k < KU; ++k) {
                            const float dx = q0.x - xh[k], dy = q0.y - yh[k], dz = q0.z - zh[k];
                            float r2 = fmaf(dx, dx, eps2);
                            r2 = fmaf(dy, dy, r2);
                            r2 = fmaf(dz, dz, r2);
                            const float ri = rsqrt_approx_g(r2);
                            const float qdx = fmaf(qa.x, dx, fmaf(qa.w, dy, qb.x * dz));
                            const float qdy = fmaf(qa.w, dx, fmaf(qa.y, dy, qb.y * dz));
                            const float qdz = fmaf(qb.x, dx, fmaf(qb.y, dy, qa.z * dz));
                            const float sq = fmaf(qdx, dx, fmaf(qdy, dy, fmaf(qdz, dz, qb.z)));
                            const float ri2 = ri * ri, ri3 = ri2 * ri, ri5 = ri3 * ri2;
                            const float tq = sq * ri5;
                            const float A = fmaf(tq * ri2, 2.5f, q0.w * ri3);
                            g[k][3] = fmaf(A, dx, fmaf(-ri5, qdx, g[k][3]));
                            g[k][4] = fmaf(A, dy, fmaf(-ri5, qdy, g[k][4]));
                            g[k][5] = fmaf(A, dz, fmaf(-ri5, qdz, g[k][5]));
                            g[k][6] = fmaf(-0.5f, tq, fmaf(-q0.w, ri, g[k][6]));
                        }
                    }
                    since += j1 - j0;
                    if (since >= kFlushG) flush();
                }
            }
            if (active) flush();
            __syncthreads();
            if (active && js == 0) {
#pragma unroll
                for (int k = 0; k < KU; ++k) {
                    const int ii = li + k * S;
                    if (ii >= nip) continue;
                    const int gi = wd.i_begin + ipass + ii;
                    double r[7] = {0, 0, 0, 0, 0, 0, 0};
                    for (int q = 0; q < n_js; ++q) {
                        const int src = q * S + li;
#pragma unroll
                        for (int c = 0; c < 7; ++c) r[c] += (double)s.acc[k][c][src].x + (double)s.acc[k][c][src].y;
                    }
                    const Accp a = p.epi_acc64[gi];
                    const double G = p.G;
                    p.out_acorr[gi] = Accp{2.0 * r[0], 2.0 * r[1], 2.0 * r[2], 0.0};
                    p.out_accp[gi] = Accp{a.x + G * r[3], a.y + G * r[4], a.z + G * r[5], G * r[6]};
                    p.out_nnb[gi] = 0;
                }
            }
        }
    }
}

constexpr int kKuG = 2;  // i per thread

}  // namespace

cudaError_t launch_gradient(const Params& p, cudaStream_t s, int num_sms) {
    cudaError_t e = cudaMemsetAsync(p.queue_head, 0, sizeof(int32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.n_retest, 0, sizeof(int32_t), s);
    if (e != cudaSuccess || p.n_walk <= 0) return e;
    static int per_sm = 0;
    if (per_sm == 0) {
        e = cudaFuncSetAttribute(gradient_kernel<kKuG>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(SmemG<kKuG>));
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gradient_kernel<kKuG>, kThreadsG,
                                                          sizeof(SmemG<kKuG>));
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    int grid = num_sms * per_sm;
    if (grid > p.n_walk) grid = p.n_walk;
    gradient_kernel<kKuG><<<grid, kThreadsG, sizeof(SmemG<kKuG>), s>>>(p);
    return cudaGetLastError();
}

}  // namespace pgf
