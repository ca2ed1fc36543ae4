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
// threads form floor(256 / ceil(n_i / 2)) j-slices.  The pair arithmetic is
// packed FP32x2 over pairs of j.  Threads stage 256-entry
// EPJ tiles (positions as walk-relative (hi, lo) pairs from the FP32 split
// arrays, accelerations as (hi, lo) pairs) and 256-entry SPJ tiles in shared
// memory.  Pair arithmetic is FP32 with both halves, so dr and da are accurate
// to an ulp of themselves for close pairs; partial sums are flushed into
// (hi, lo) FP32 accumulators and the slices are combined in FP64.
#include "pgf_internal.cuh"

namespace pgf {
namespace {

constexpr int kThreadsG = 256;
constexpr int kTileEPG = 256;
constexpr int kTileSPG = 256;  // as many pairs per tile as an EP tile
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

// Double-float helpers: a value is an FP32 pair (h, l) with h + l exact to
// about 2^-48 relative.  two_prod_g is exact with one FMA.
__device__ __forceinline__ void two_prod_g(float a, float b, float& p, float& e) {
    p = a * b;
    e = fmaf(a, b, -p);
}

// (x_j - x_i) as a double-float from both operands' (hi, lo) halves; the i
// halves are passed negated.
__device__ __forceinline__ void df_diff(float jh, float jl, float nih, float nil, float& h, float& l) {
    float s, e;
    two_sum_g(jh, nih, s, e);
    two_sum_g(s, e + (jl + nil), h, l);
}

__device__ __forceinline__ void flush_into(float2& v, float x) {
    float e;
    two_sum_g(v.x, x, v.x, e);
    v.y += e;
}

// Far pairs with r^2 and 1/r carried beyond FP32 (the compensated option).
// r^2 = dx^2 + dy^2 + dz^2 + eps^2 as a (hi, lo) pair: exact squares by FMA
// and error-free sums (the Dot2 scheme of Ogita, Rump and Oishi, 2005).  1/r
// from y = rsqrt(hi) and the residual t = 1 - r^2 y^2, evaluated with the
// exact square of y, so that r^-3 = y^3 (1 + 1.5 t) and r^-2 = y^2 (1 + t)
// to O(t^2) (t is a few 2^-23).  Gives m r^-3 and r^-2.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// s = fl(a + b) and the exact error a + b - s (Knuth's two-sum), packed.
__device__ __forceinline__ float2 two_sum2_err(float2 a, float2 b, float2& s) {
    s = __fadd2_rn(a, b);
    const float2 bb = __fadd2_rn(s, neg2(a));
    const float2 ab = __fadd2_rn(s, neg2(bb));
    return __fadd2_rn(__fadd2_rn(a, neg2(ab)), __fadd2_rn(b, neg2(bb)));
}

__device__ __forceinline__ void far_r3_compensated(float2 dx, float2 dy, float2 dz, float2 e2, float2 M, float rcut2,
                                                   float2& mr3, float2& ri2) {
    const float2 px = __fmul2_rn(dx, dx), py = __fmul2_rn(dy, dy), pz = __fmul2_rn(dz, dz);
    const float2 ex = __ffma2_rn(dx, dx, neg2(px));
    const float2 ey = __ffma2_rn(dy, dy, neg2(py));
    const float2 ez = __ffma2_rn(dz, dz, neg2(pz));
    float2 s1, hi;
    const float2 c1 = two_sum2_err(px, py, s1);
    const float2 c2 = two_sum2_err(s1, pz, hi);
    // r^2 = hi + lo with |lo| of order ulp(hi)
    const float2 lo = __fadd2_rn(__fadd2_rn(__fadd2_rn(ex, ey), __fadd2_rn(ez, e2)), __fadd2_rn(c1, c2));
    // far pairs have r >= r_out; the clamp only guards rounding at the edge
    const float2 y = make_float2(rsqrt_approx_g(fmaxf(hi.x, rcut2)), rsqrt_approx_g(fmaxf(hi.y, rcut2)));
    const float2 h = __fmul2_rn(y, y);
    const float2 hl = __ffma2_rn(y, y, neg2(h));
    float2 t = __ffma2_rn(neg2(hi), h, make_float2(1.f, 1.f));
    t = __ffma2_rn(neg2(hi), hl, t);
    t = __ffma2_rn(neg2(lo), h, t);
    const float2 m3 = __fmul2_rn(__fmul2_rn(M, y), h);
    mr3 = __ffma2_rn(m3, __fmul2_rn(t, make_float2(1.5f, 1.5f)), m3);
    ri2 = __ffma2_rn(h, t, __fadd2_rn(h, hl));
}

// KU i-particles per thread: i = li + k S (k < KU) of a pass of up to
// 256 KU i, with S = ceil(n_i / KU) threads per j-slice.  Tiles are stored
// as interleaved pairs of j, so that one FP32x2 instruction evaluates two
// pairs (the FMA pipe throughput is the same, the issue slots halve).
// EPJ pair: P = (xh, yh | zh, m | xl, yl | zl, -) and A = (axh, ayh | azh,
// axl | ayl, azl), each field as (j0, j1).  SPJ pair: (x, y | z, m | -Qxx,
// -Qyy | -Qzz, -Qxy | -Qxz, -Qyz | -c, -) with c = -tr(q) eps^2, so that
// the quadrupole terms need no negation.
constexpr float kDummyPosG = 1e15f;

template <int KU>
struct SmemGP {
    float4 P[kTileEPG / 2][4];
    float4 A[kTileEPG / 2][3];
    float4 S[kTileSPG / 2][6];
    // Near entries of the EP tile at their own index: (xh, yh, zh, m),
    // (xl, yl, zl, -), (axh, ayh, azh, -), (axl, ayl, azl, -); which entries
    // are near: one bit each.
    float4 N[kTileEPG][4];
    unsigned nmask[kTileEPG / 32];
    float2 acc[KU][7][kThreadsG];
    int w;
};

template <int KU, bool CMP>
__global__ __launch_bounds__(kThreadsG, 2) void gradient_kernel_pk(Params p) {
    if (p.input_err && *p.input_err) return;  // the inputs failed their check: run nothing
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SmemGP<KU>& s = *reinterpret_cast<SmemGP<KU>*>(smem_raw);
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
        // Near entries (possibly within r_out of an i of the walk's box):
        // their pairs run in the near loop below.  Inside r_out the distance
        // is clamped to r_out, and da - 3 (dr.da) / r_out^2 dr cancels for
        // pairs at r_out / sqrt(3) with da along dr (close binary companions);
        // those pairs are evaluated in double-float arithmetic with
        // kdf = 3 / r_out^2 and r3c = r_out^-3 formed in FP64 here.
        const float rc = sqrtf(rcut2);
        const float hmax = fmaxf(wd.hx, fmaxf(wd.hy, wd.hz));
        const double kd = 3.0 / wd.rcut2;
        const float kdh = (float)kd, kdl = (float)(kd - (double)kdh);
        const float r3c = (float)(1.0 / (wd.rcut2 * sqrt(wd.rcut2)));
        for (int ipass = 0; ipass < wd.n_i; ipass += kThreadsG * KU) {
            const int nip = min(kThreadsG * KU, wd.n_i - ipass);
            const int S = (nip + KU - 1) / KU;
            const int n_js = kThreadsG / S;
            const int js = tid / S;
            const int li = tid - js * S;
            const bool active = js < n_js;
            // (-x_i, -x_i) operands: position and acceleration, hi and lo
            float2 nxh[KU], nyh[KU], nzh[KU], nxl[KU], nyl[KU], nzl[KU];
            float2 nah[KU][3], nal[KU][3];
#pragma unroll
            for (int k = 0; k < KU; ++k) {
                float v[12] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                const int ii = li + k * S;
                if (active && ii < nip) {
                    const int gi = wd.i_begin + ipass + ii;
                    const EpiDev e = p.epi[gi];
                    const double d[3] = {e.x - wd.cx, e.y - wd.cy, e.z - wd.cz};
                    const Accp a = p.epi_acc64[gi];
                    const double aa[3] = {a.x, a.y, a.z};
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        v[c] = (float)d[c];
                        v[3 + c] = (float)(d[c] - (double)v[c]);
                        v[6 + c] = (float)aa[c];
                        v[9 + c] = (float)(aa[c] - (double)v[6 + c]);
                    }
                }
                nxh[k] = make_float2(-v[0], -v[0]);
                nyh[k] = make_float2(-v[1], -v[1]);
                nzh[k] = make_float2(-v[2], -v[2]);
                nxl[k] = make_float2(-v[3], -v[3]);
                nyl[k] = make_float2(-v[4], -v[4]);
                nzl[k] = make_float2(-v[5], -v[5]);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    nah[k][c] = make_float2(-v[6 + c], -v[6 + c]);
                    nal[k][c] = make_float2(-v[9 + c], -v[9 + c]);
                }
            }
#pragma unroll
            for (int k = 0; k < KU; ++k)
#pragma unroll
                for (int q = 0; q < 7; ++q) s.acc[k][q][tid] = make_float2(0.f, 0.f);
            // Pair accumulators: acorr x, y, z, SP acc x, y, z, minus SP pot.
            float2 g[KU][7];
#pragma unroll
            for (int k = 0; k < KU; ++k)
#pragma unroll
                for (int q = 0; q < 7; ++q) g[k][q] = make_float2(0.f, 0.f);
            int since = 0;
            auto flush = [&]() {
#pragma unroll
                for (int k = 0; k < KU; ++k)
#pragma unroll
                    for (int q = 0; q < 7; ++q) {
                        const float x = g[k][q].x + g[k][q].y;
                        flush_into(s.acc[k][q][tid], q == 6 ? -x : x);
                        g[k][q] = make_float2(0.f, 0.f);
                    }
                since = 0;
            };
            // The acorr partial sums alone (the compensated mode flushes them
            // every 8 j pairs: the sum over j cancels, and long FP32 partial
            // sums would round away what the compensated terms keep).
            auto flush_acorr = [&]() {
#pragma unroll
                for (int k = 0; k < KU; ++k)
#pragma unroll
                    for (int q = 0; q < 3; ++q) {
                        flush_into(s.acc[k][q][tid], g[k][q].x + g[k][q].y);
                        g[k][q] = make_float2(0.f, 0.f);
                    }
            };
            const float2 e2 = make_float2(eps2, eps2);
            // EPJ tiles: the gradient correction of every pair.
            for (int t = 0; t < wd.n_epj; t += kTileEPG) {
                const int nt = min(kTileEPG, wd.n_epj - t);
                __syncthreads();
                bool near = false;
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
                    // Conservative box test (0.2% and absolute margins over r_out).
                    const float ex = fmaxf(fabsf(hx) - wd.hx, 0.f);
                    const float ey = fmaxf(fabsf(hy) - wd.hy, 0.f);
                    const float ez = fmaxf(fabsf(hz) - wd.hz, 0.f);
                    const float dist2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                    const float dmax = fmaxf(fabsf(hx), fmaxf(fabsf(hy), fabsf(hz)));
                    const float Rm = rc * 1.002f + 1e-6f * (dmax + hmax);
                    near = !(dist2 > Rm * Rm);
                    if (near) {
                        s.N[tid][0] = make_float4(hx, hy, hz, r.m);
                        s.N[tid][1] = make_float4(lx, ly, lz, 0.f);
                        s.N[tid][2] = make_float4(a.xh, a.yh, a.zh, 0.f);
                        s.N[tid][3] = make_float4(a.xl, a.yl, a.zl, 0.f);
                    }
                    float* P = reinterpret_cast<float*>(&s.P[tid >> 1][0]) + (tid & 1);
                    P[0] = hx;
                    P[2] = hy;
                    P[4] = hz;
                    P[6] = near ? 0.f : r.m;  // near pairs run in the near loop
                    P[8] = lx;
                    P[10] = ly;
                    P[12] = lz;
                    P[14] = 0.f;
                    float* A = reinterpret_cast<float*>(&s.A[tid >> 1][0]) + (tid & 1);
                    A[0] = a.xh;
                    A[2] = a.yh;
                    A[4] = a.zh;
                    A[6] = a.xl;
                    A[8] = a.yl;
                    A[10] = a.zl;
                } else if (tid == nt && (nt & 1)) {
                    // massless partner of the last entry
                    float* P = reinterpret_cast<float*>(&s.P[tid >> 1][0]) + 1;
                    float* A = reinterpret_cast<float*>(&s.A[tid >> 1][0]) + 1;
                    for (int u = 0; u < 16; u += 2) P[u] = 0.f;
                    for (int u = 0; u < 12; u += 2) A[u] = 0.f;
                }
                {
                    const unsigned bn = __ballot_sync(0xffffffffu, near);
                    if ((tid & 31) == 0 && tid < kTileEPG) s.nmask[tid >> 5] = bn;
                }
                __syncthreads();
                if (active) {
                    const int np = (nt + 1) >> 1;
                    const int pn = (np + n_js - 1) / n_js;
                    const int j0 = min(np, js * pn), j1 = min(np, j0 + pn);
                    for (int j = j0; j < j1; ++j) {
                        const float4 p0 = s.P[j][0], p1 = s.P[j][1], p2 = s.P[j][2], p3 = s.P[j][3];
                        const float4 a0 = s.A[j][0], a1 = s.A[j][1], a2 = s.A[j][2];
                        const float2 Xh = make_float2(p0.x, p0.y), Yh = make_float2(p0.z, p0.w);
                        const float2 Zh = make_float2(p1.x, p1.y), M = make_float2(p1.z, p1.w);
                        const float2 Xl = make_float2(p2.x, p2.y), Yl = make_float2(p2.z, p2.w);
                        const float2 Zl = make_float2(p3.x, p3.y);
                        const float2 AXh = make_float2(a0.x, a0.y), AYh = make_float2(a0.z, a0.w);
                        const float2 AZh = make_float2(a1.x, a1.y), AXl = make_float2(a1.z, a1.w);
                        const float2 AYl = make_float2(a2.x, a2.y), AZl = make_float2(a2.z, a2.w);
#pragma unroll
                        for (int k = 0; k < KU; ++k) {
                            // x_j - x_i and a_j - a_i from both halves
                            const float2 dx = __fadd2_rn(__fadd2_rn(Xh, nxh[k]), __fadd2_rn(Xl, nxl[k]));
                            const float2 dy = __fadd2_rn(__fadd2_rn(Yh, nyh[k]), __fadd2_rn(Yl, nyl[k]));
                            const float2 dz = __fadd2_rn(__fadd2_rn(Zh, nzh[k]), __fadd2_rn(Zl, nzl[k]));
                            const float2 dax = __fadd2_rn(__fadd2_rn(AXh, nah[k][0]), __fadd2_rn(AXl, nal[k][0]));
                            const float2 day = __fadd2_rn(__fadd2_rn(AYh, nah[k][1]), __fadd2_rn(AYl, nal[k][1]));
                            const float2 daz = __fadd2_rn(__fadd2_rn(AZh, nah[k][2]), __fadd2_rn(AZl, nal[k][2]));
                            float2 ri2, mr3;
                            if constexpr (CMP) {
                                far_r3_compensated(dx, dy, dz, e2, M, rcut2, mr3, ri2);
                            } else {
                                float2 r2 = __ffma2_rn(dx, dx, e2);
                                r2 = __ffma2_rn(dy, dy, r2);
                                r2 = __ffma2_rn(dz, dz, r2);
                                const float2 ri = make_float2(rsqrt_approx_g(fmaxf(r2.x, rcut2)),
                                                              rsqrt_approx_g(fmaxf(r2.y, rcut2)));
                                ri2 = __fmul2_rn(ri, ri);
                                mr3 = __fmul2_rn(__fmul2_rn(M, ri), ri2);
                            }
                            const float2 drda = __ffma2_rn(dx, dax, __ffma2_rn(dy, day, __fmul2_rn(dz, daz)));
                            // -alpha = -3 (dr.da) / r^2
                            const float2 nal_ = __fmul2_rn(__fmul2_rn(drda, ri2), make_float2(-3.f, -3.f));
                            g[k][0] = __ffma2_rn(mr3, __ffma2_rn(nal_, dx, dax), g[k][0]);
                            g[k][1] = __ffma2_rn(mr3, __ffma2_rn(nal_, dy, day), g[k][1]);
                            g[k][2] = __ffma2_rn(mr3, __ffma2_rn(nal_, dz, daz), g[k][2]);
                        }
                        if constexpr (CMP) {
                            if (((j - j0) & 7) == 7) flush_acorr();
                        }
                    }
                    since += 2 * (j1 - j0);
                    // Near entries, each handled by slice (index mod n_js).
                    for (int wv = 0; wv < kTileEPG / 32; ++wv) {
                        unsigned m = s.nmask[wv];
                        while (m) {
                            const int e = wv * 32 + __ffs(m) - 1;
                            m &= m - 1;
                            if (e % n_js != js) continue;
                            const float4 q0 = s.N[e][0], q1 = s.N[e][1], q2 = s.N[e][2], q3 = s.N[e][3];
#pragma unroll
                            for (int k = 0; k < KU; ++k) {
                                if (li + k * S >= nip) continue;
                                // dr and da from both halves, as the packed loop forms them
                                const float d0 = (q0.x + nxh[k].x) + (q1.x + nxl[k].x);
                                const float d1 = (q0.y + nyh[k].x) + (q1.y + nyl[k].x);
                                const float d2 = (q0.z + nzh[k].x) + (q1.z + nzl[k].x);
                                const float r2 = fmaf(d0, d0, fmaf(d1, d1, fmaf(d2, d2, eps2)));
                                float v[3], mr3;
                                if (r2 < rcut2) {
                                    // clamped: v = da - (3 / r_out^2)(dr.da) dr in double-float
                                    float dh[3], dl[3], ah[3], al[3];
                                    df_diff(q0.x, q1.x, nxh[k].x, nxl[k].x, dh[0], dl[0]);
                                    df_diff(q0.y, q1.y, nyh[k].x, nyl[k].x, dh[1], dl[1]);
                                    df_diff(q0.z, q1.z, nzh[k].x, nzl[k].x, dh[2], dl[2]);
                                    df_diff(q2.x, q3.x, nah[k][0].x, nal[k][0].x, ah[0], al[0]);
                                    df_diff(q2.y, q3.y, nah[k][1].x, nal[k][1].x, ah[1], al[1]);
                                    df_diff(q2.z, q3.z, nah[k][2].x, nal[k][2].x, ah[2], al[2]);
                                    float sh = 0.f, sl = 0.f;
#pragma unroll
                                    for (int c = 0; c < 3; ++c) {
                                        float pp, pe, t1, t2;
                                        two_prod_g(dh[c], ah[c], pp, pe);
                                        pe = fmaf(dh[c], al[c], fmaf(dl[c], ah[c], pe));
                                        two_sum_g(sh, pp, t1, t2);
                                        sh = t1;
                                        sl += t2 + pe;
                                    }
                                    float alh, ale;
                                    two_prod_g(kdh, sh, alh, ale);
                                    ale = fmaf(kdh, sl, fmaf(kdl, sh, ale));
#pragma unroll
                                    for (int c = 0; c < 3; ++c) {
                                        float qh, qe, vh, ve;
                                        two_prod_g(alh, dh[c], qh, qe);
                                        qe = fmaf(alh, dl[c], fmaf(ale, dh[c], qe));
                                        two_sum_g(ah[c], -qh, vh, ve);
                                        v[c] = vh + (ve + (al[c] - qe));
                                    }
                                    mr3 = q0.w * r3c;
                                } else {
                                    const float e0 = (q2.x + nah[k][0].x) + (q3.x + nal[k][0].x);
                                    const float e1 = (q2.y + nah[k][1].x) + (q3.y + nal[k][1].x);
                                    const float e2_ = (q2.z + nah[k][2].x) + (q3.z + nal[k][2].x);
                                    float ri2;
                                    if constexpr (CMP) {
                                        float2 m2, r22;
                                        far_r3_compensated(make_float2(d0, d0), make_float2(d1, d1),
                                                           make_float2(d2, d2), make_float2(eps2, eps2),
                                                           make_float2(q0.w, q0.w), rcut2, m2, r22);
                                        mr3 = m2.x;
                                        ri2 = r22.x;
                                    } else {
                                        const float ri = rsqrt_approx_g(r2);
                                        ri2 = ri * ri;
                                        mr3 = (q0.w * ri) * ri2;
                                    }
                                    const float nl3 = -3.f * (fmaf(d0, e0, fmaf(d1, e1, d2 * e2_)) * ri2);
                                    v[0] = fmaf(nl3, d0, e0);
                                    v[1] = fmaf(nl3, d1, e1);
                                    v[2] = fmaf(nl3, d2, e2_);
                                }
                                g[k][0].x = fmaf(mr3, v[0], g[k][0].x);
                                g[k][1].x = fmaf(mr3, v[1], g[k][1].x);
                                g[k][2].x = fmaf(mr3, v[2], g[k][2].x);
                            }
                            ++since;
                        }
                    }
                    if (since >= kFlushG) flush();
                }
            }
            // SPJ tiles: the quadrupole force.
            for (int t = 0; t < wd.n_spj; t += kTileSPG) {
                const int nt = min(kTileSPG, wd.n_spj - t);
                __syncthreads();
                if (tid < nt) {
                    const int id = p.id_spj[wd.spj_begin + t + tid];
                    const SpjF32 r = p.spj32[id];
                    float* f = reinterpret_cast<float*>(&s.S[tid >> 1][0]) + (tid & 1);
                    f[0] = (r.xh - chx) + (r.xl - clx);
                    f[2] = (r.yh - chy) + (r.yl - cly);
                    f[4] = (r.zh - chz) + (r.zl - clz);
                    f[6] = r.m;
                    f[8] = -r.Q[0];
                    f[10] = -r.Q[1];
                    f[12] = -r.Q[2];
                    f[14] = -r.Q[3];
                    f[16] = -r.Q[4];
                    f[18] = -r.Q[5];
                    f[20] = r.tr * eps2;
                    f[22] = 0.f;
                } else if (tid == nt && (nt & 1)) {
                    // massless, moment-free partner far away
                    float* f = reinterpret_cast<float*>(&s.S[tid >> 1][0]) + 1;
                    f[0] = f[2] = f[4] = kDummyPosG;
                    for (int u = 6; u < 24; u += 2) f[u] = 0.f;
                }
                __syncthreads();
                if (active) {
                    const int np = (nt + 1) >> 1;
                    const int ps = (np + n_js - 1) / n_js;
                    const int j0 = min(np, js * ps), j1 = min(np, j0 + ps);
                    const float2 km25 = make_float2(-2.5f, -2.5f), km05 = make_float2(-0.5f, -0.5f);
                    for (int j = j0; j < j1; ++j) {
                        const float4 w0 = s.S[j][0], w1 = s.S[j][1], w2 = s.S[j][2];
                        const float4 w3 = s.S[j][3], w4 = s.S[j][4], w5 = s.S[j][5];
                        const float2 X = make_float2(w0.x, w0.y), Y = make_float2(w0.z, w0.w);
                        const float2 Z = make_float2(w1.x, w1.y), M = make_float2(w1.z, w1.w);
                        const float2 Qxx = make_float2(w2.x, w2.y), Qyy = make_float2(w2.z, w2.w);
                        const float2 Qzz = make_float2(w3.x, w3.y), Qxy = make_float2(w3.z, w3.w);
                        const float2 Qxz = make_float2(w4.x, w4.y), Qyz = make_float2(w4.z, w4.w);
                        const float2 C = make_float2(w5.x, w5.y);
#pragma unroll
                        for (int k = 0; k < KU; ++k) {
                            const float2 dx = __fadd2_rn(X, nxh[k]);
                            const float2 dy = __fadd2_rn(Y, nyh[k]);
                            const float2 dz = __fadd2_rn(Z, nzh[k]);
                            float2 r2 = __ffma2_rn(dx, dx, e2);
                            r2 = __ffma2_rn(dy, dy, r2);
                            r2 = __ffma2_rn(dz, dz, r2);
                            const float2 ri = make_float2(rsqrt_approx_g(r2.x), rsqrt_approx_g(r2.y));
                            // with -Q and -c: u = d.(-Q).d - c = -(d.Q.d + c), t = u / r^5
                            const float2 qdx = __ffma2_rn(Qxx, dx, __ffma2_rn(Qxy, dy, __fmul2_rn(Qxz, dz)));
                            const float2 qdy = __ffma2_rn(Qxy, dx, __ffma2_rn(Qyy, dy, __fmul2_rn(Qyz, dz)));
                            const float2 qdz = __ffma2_rn(Qxz, dx, __ffma2_rn(Qyz, dy, __fmul2_rn(Qzz, dz)));
                            const float2 sq = __ffma2_rn(qdx, dx, __ffma2_rn(qdy, dy, __ffma2_rn(qdz, dz, C)));
                            const float2 ri2 = __fmul2_rn(ri, ri);
                            const float2 ri3 = __fmul2_rn(ri2, ri);
                            const float2 ri5 = __fmul2_rn(ri3, ri2);
                            const float2 tq = __fmul2_rn(sq, ri5);
                            const float2 A = __ffma2_rn(__fmul2_rn(tq, ri2), km25, __fmul2_rn(M, ri3));
                            g[k][3] = __ffma2_rn(A, dx, __ffma2_rn(ri5, qdx, g[k][3]));
                            g[k][4] = __ffma2_rn(A, dy, __ffma2_rn(ri5, qdy, g[k][4]));
                            g[k][5] = __ffma2_rn(A, dz, __ffma2_rn(ri5, qdz, g[k][5]));
                            g[k][6] = __ffma2_rn(tq, km05, __ffma2_rn(M, ri, g[k][6]));
                        }
                    }
                    since += 2 * (j1 - j0);
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
                    // a_i once: parts of a split walk add their pairs only
                    const Accp a = wd.part == 0 ? p.epi_acc64[gi] : Accp{0.0, 0.0, 0.0, 0.0};
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

template <bool CMP>
cudaError_t launch_gradient_t(const Params& p, cudaStream_t s, int num_sms) {
    static int per_sm = 0;
    cudaError_t e;
    if (per_sm == 0) {
        e = cudaFuncSetAttribute(gradient_kernel_pk<kKuG, CMP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(SmemGP<kKuG>));
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gradient_kernel_pk<kKuG, CMP>, kThreadsG,
                                                          sizeof(SmemGP<kKuG>));
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    int grid = num_sms * per_sm;
    if (grid > p.n_walk) grid = p.n_walk;
    gradient_kernel_pk<kKuG, CMP><<<grid, kThreadsG, sizeof(SmemGP<kKuG>), s>>>(p);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gradient(const Params& p, cudaStream_t s, int num_sms) {
    cudaError_t e = cudaMemsetAsync(p.queue_head, 0, sizeof(int32_t), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.n_retest, 0, sizeof(int32_t), s);
    if (e != cudaSuccess || p.n_walk <= 0) return e;
    return p.gr_compensated ? launch_gradient_t<true>(p, s, num_sms) : launch_gradient_t<false>(p, s, num_sms);
}

}  // namespace pgf
