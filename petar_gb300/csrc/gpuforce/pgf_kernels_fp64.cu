// Plain FP64 soft-force kernel: the drop-in baseline the mixed-precision
// kernel is measured against.
//
// Same arithmetic as the reference's FP64 functors (src/soft_force.hpp:53-71
// for EP-EP with the linear cutoff, :174-195 for the EP-SP quadrupole) in
// double precision throughout, one thread per i-particle, j tiles staged in
// shared memory, walks taken from the length-sorted work queue.  The
// neighbour test uses the oracle's exact evaluation order, so its counts are
// bit-exact.
#include "pgf_internal.cuh"

namespace pgf {
namespace {

constexpr int kT = 128;  // threads per block = i per chunk = j per tile

__global__ __launch_bounds__(kT) void fp64_kernel(Params p) {
    if (p.input_err && *p.input_err) return;  // the inputs failed their check: run nothing
    __shared__ double sx[kT], sy[kT], sz[kT], sm[kT], srs[kT];
    __shared__ double sq[6][kT];
    __shared__ int s_w;
    const int tid = threadIdx.x;
    const double eps2 = p.eps2;
    const int n_walk = walk_count(p);
    for (;;) {
        if (tid == 0) s_w = atomicAdd(p.queue_head, 1);
        __syncthreads();
        const int wq = s_w;
        __syncthreads();
        if (wq >= n_walk) break;
        const WalkDesc wd = p.walks[p.order[wq]];
        const double rcut2 = wd.rcut2;
        for (int ic = 0; ic < wd.n_i; ic += kT) {
            const int li = ic + tid;
            const bool valid = li < wd.n_i;
            double xi = 0, yi = 0, zi = 0, rsi = 0;
            if (valid) {
                const EpiDev e = p.epi[wd.i_begin + li];
                xi = e.x;
                yi = e.y;
                zi = e.z;
                rsi = e.rs;
            }
            double ax = 0, ay = 0, az = 0, pe = 0;
            int nnb = 0;
            for (int t0 = 0; t0 < wd.n_epj; t0 += kT) {
                const int nt = min(kT, wd.n_epj - t0);
                __syncthreads();
                if (tid < nt) {
                    const int id = p.id_epj[wd.epj_begin + t0 + tid];
                    const EpjMix j = p.epj[id];
                    sx[tid] = j.x;
                    sy[tid] = j.y;
                    sz[tid] = j.z;
                    sm[tid] = p.epj_m64[id];
                    srs[tid] = p.epj_rs64[id];
                }
                __syncthreads();
                if (valid) {
                    for (int k = 0; k < nt; ++k) {
                        const double dx = __dsub_rn(xi, sx[k]);
                        const double dy = __dsub_rn(yi, sy[k]);
                        const double dz = __dsub_rn(zi, sz[k]);
                        const double r2 =
                            __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
                        const double r2e = __dadd_rn(r2, eps2);
                        const double rs = rsi > srs[k] ? rsi : srs[k];
                        nnb += r2e < __dmul_rn(rs, rs) ? 1 : 0;
                        const double r2c = r2e > rcut2 ? r2e : rcut2;
                        const double ri = rsqrt(r2c);
                        const double mr = sm[k] * ri;
                        const double mr3 = mr * ri * ri;
                        ax -= mr3 * dx;
                        ay -= mr3 * dy;
                        az -= mr3 * dz;
                        pe -= mr;
                    }
                }
            }
            double bx = 0, by = 0, bz = 0, ps = 0;
            for (int t0 = 0; t0 < wd.n_spj; t0 += kT) {
                const int nt = min(kT, wd.n_spj - t0);
                __syncthreads();
                if (tid < nt) {
                    const int id = p.id_spj[wd.spj_begin + t0 + tid];
                    const SpjMix j = p.spj[id];
                    const SpjQ64 q = p.spj_q64[id];
                    sx[tid] = j.x;
                    sy[tid] = j.y;
                    sz[tid] = j.z;
                    sm[tid] = q.m;
                    for (int c = 0; c < 6; ++c) sq[c][tid] = q.q[c];
                }
                __syncthreads();
                if (valid) {
                    for (int k = 0; k < nt; ++k) {
                        const double rx = xi - sx[k];
                        const double ry = yi - sy[k];
                        const double rz = zi - sz[k];
                        const double r2 = rx * rx + ry * ry + rz * rz + eps2;
                        const double qxx = sq[0][k], qyy = sq[1][k], qzz = sq[2][k];
                        const double qxy = sq[3][k], qxz = sq[4][k], qyz = sq[5][k];
                        const double tr = qxx + qyy + qzz;
                        const double qrx = qxx * rx + qxy * ry + qxz * rz;
                        const double qry = qyy * ry + qyz * rz + qxy * rx;
                        const double qrz = qzz * rz + qxz * rx + qyz * ry;
                        const double qrr = qrx * rx + qry * ry + qrz * rz;
                        const double r_inv = rsqrt(r2);
                        const double r2_inv = r_inv * r_inv;
                        const double r3_inv = r2_inv * r_inv;
                        const double r5_inv = r2_inv * r3_inv * 1.5;
                        const double qrr_r5 = r5_inv * qrr;
                        const double qrr_r7 = r2_inv * qrr_r5;
                        const double A = sm[k] * r3_inv - tr * r5_inv + 5.0 * qrr_r7;
                        const double B = -2.0 * r5_inv;
                        bx -= A * rx + B * qrx;
                        by -= A * ry + B * qry;
                        bz -= A * rz + B * qrz;
                        ps -= sm[k] * r_inv - 0.5 * tr * r3_inv + qrr_r5;
                    }
                }
            }
            if (valid) {
                const double G = p.G;
                const int gi = wd.i_begin + li;
                p.out_accp[gi] = Accp{G * ax + G * bx, G * ay + G * by, G * az + G * bz, G * pe + G * ps};
                p.out_nnb[gi] = nnb;
            }
        }
    }
}

}  // namespace

cudaError_t launch_fp64(const Params& p, cudaStream_t s, int num_sms) {
    cudaError_t e = cudaMemsetAsync(p.queue_head, 0, sizeof(int32_t), s);
    if (e != cudaSuccess) return e;
    if (p.n_walk <= 0) return cudaSuccess;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fp64_kernel, kT, 0);
    if (e != cudaSuccess) return e;
    int grid = num_sms * (per_sm > 0 ? per_sm : 1);
    if (grid > p.n_walk) grid = p.n_walk;
    fp64_kernel<<<grid, kT, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace pgf
