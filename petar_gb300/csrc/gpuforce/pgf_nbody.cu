// Device-resident soft-force step: tree, interaction lists, force, kicks and
// drifts without a host round trip, so a run of steps is captured in one CUDA
// graph.
//
// In PeTar the tree step of every particle goes through the host:
// treeSoftForce (src/petar.hpp:879-907) asks FDPS to build the tree and walk
// it, and FDPS hands the lists to the GPU functor group by group; kickOne
// (src/petar.hpp:1198-1212) and driftSingle (src/petar.hpp:1326-1340) update
// velocities and positions on the host between evaluations.  Here the same
// cycle runs on the device for singles without a hard part:
//
//   kick(dt/2) + drift(dt)  ->  tree + lists  ->  force  ->  kick(dt/2)
//
// The tree and the lists follow the host list builder
// (csrc/harness/walk_builder.cpp, the stand-in for FDPS's
// TreeForForceLong<...>::QuadrupoleWithSymmetrySearch) step by step, and this
// file is compiled without FMA contraction, so the device lists equal the
// host builder's entry for entry:
//   * Morton keys of 21 bits per axis inside the cubic root cell, sorted
//     stably (CUB radix sort) with the particle index as value;
//   * an octree built level by level: a cell with more than n_leaf_limit
//     particles (and above level 21) splits into its non-empty octants, the
//     children of a level numbered in their parents' order (breadth-first
//     numbering, children of a cell contiguous);
//   * moments bottom-up: a leaf sums its particles in sorted order, a parent
//     combines its children in child order (mass, mass moment, centre of
//     mass, second moment with the parallel-axis term), plus the particle box
//     and the r_search-expanded box;
//   * i-groups: the topmost cells with at most n_group_limit particles (or
//     leaves), in Morton order;
//   * per group a depth-first walk that opens a cell when the distance from
//     the group's box to the cell's centre of mass is within side / theta or
//     when the r_search-expanded boxes overlap (symmetric search); opened
//     leaves give their particles as EPJ, unopened cells their moments as SPJ.
// Lists are built in two passes (count, scan, fill) into arrays sized at
// creation with room to grow; a build that would overflow any capacity sets
// an error bit, runs no force kernel and the host reports PGF_ERR_CAPACITY.
//
// The walks run as one thread per (group, pair of frontier cells), taken a
// warp at a time from a counter.  The frontier cells are the topmost cells
// with at most n / 512 particles (at least n_group_limit) (or
// leaves); they partition the particles in Morton order, so the depth-first
// list of a group is the concatenation, in frontier order, of the lists of
// the frontier subtrees (a cell above the frontier that the group does not
// open is listed once, by the first frontier cell below it).  The opening test runs in FP32
// on rounded copies of the cell data with rigorous bounds on the rounding,
// and falls back to the FP64 test only where the bounds cannot decide, so the
// decisions, and the lists, are exactly those of the FP64 test.
#include "petar_gpuforce.h"
#include "pgf_internal.cuh"

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_select.cuh>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace pgf {
namespace {

constexpr int kMaxLevel = 21;          // 3 x 21 bits of Morton key
constexpr int kLevels = kMaxLevel + 1;  // levels 0 .. 21
constexpr int kStack = 160;            // DFS stack: 1 + 7 x 21 entries at most
constexpr int kBuckets = 256;          // work-queue cost buckets
constexpr int kLeafBins = 64;          // leaf size classes of the moments launches
constexpr int kCellBins = kLeafBins + 8 * kLevels;  // and inner cells by level and child count
constexpr int kScanThreads = 1024;

enum : int32_t { kErrCells = 1, kErrEpj = 2, kErrSpj = 4, kErrTasks = 8 };
constexpr float kU = 5.9604645e-8f;  // 2^-24, unit roundoff of FP32

struct TreeHdr {
    double root_lo[3];
    double half;
    double scale;
    double side0;
    int32_t level_begin[kLevels + 2];  // cells of level L: [level_begin[L], level_begin[L + 1])
    int32_t n_groups;
    int32_t n_fronts;  // frontier cells
    float xmax;        // bound on |coordinate| of every centre of mass and particle box
    int32_t n_walk;  // n_groups, or 0 when the build overflowed
    int32_t err;     // kErr* bits of this build
    int32_t err_sticky;
    int64_t n_epj_entries, n_spj_entries;  // list totals of this build (also when over capacity)
    unsigned long long n_epep, n_epsp;     // interactions of this build's lists
    unsigned long long total_epep, total_epsp;
    int32_t hist[kBuckets];
    int32_t cursor[kBuckets];
    int32_t cell_hist[kCellBins];    // cells by moments class
    int32_t cell_cursor[kCellBins];  // their slots in the class-ordered cell list
    int32_t sample_slot;  // next record slot of the per-step sample
    int32_t pad2;
    unsigned long long walk_cursor[2];  // next task of the count and fill passes
};

// Cell fields the walk reads.
struct __align__(32) TCell {
    double com[3];
    double crit;  // (side * side) / theta^2
    double in_lo[3], in_hi[3];
    double out_lo[3], out_hi[3];
    int32_t begin, end, first_child, n_child;
    int32_t leaf, level, parent;
    float rs_max;  // largest r_search of the cell's particles, rounded up
};
static_assert(sizeof(TCell) == 160, "TCell layout");

// Rounded (FP32) copy of the cell data for the walk's fast path.
struct __align__(16) TCellW {
    float com[3];
    float crit;
    float in_lo[3], in_hi[3];
    float out_lo[3], out_hi[3];
    int32_t begin, end, first_child, n_child;
    int32_t leaf, parent, level, pad1;
};
static_assert(sizeof(TCellW) == 96, "TCellW layout");

struct CMom {
    double m;
    double mx[3];
    double q[6];  // xx, yy, zz, xy, xz, yz about the centre of mass
};

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ double dmin(double a, double b) { return b < a ? b : a; }  // std::min
__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }  // std::max

// The same for non-NaN values on the integer pipe (GB300 runs FP64 at 1/64 of
// the FP32 rate): doubles ordered as signed 64-bit keys, -0 and +0 equal as
// the FP64 comparison sees them, ties returning a as above.
__device__ __forceinline__ int64_t order_key(double x) {
    int64_t b = __double_as_longlong(x);
    if (b == (int64_t)0x8000000000000000ull) b = 0;
    return b < 0 ? (b ^ 0x7fffffffffffffffll) : b;
}
__device__ __forceinline__ double kmin(double a, double b) { return order_key(b) < order_key(a) ? b : a; }
__device__ __forceinline__ double kmax(double a, double b) { return order_key(a) < order_key(b) ? b : a; }

__device__ __forceinline__ uint64_t spread3(uint64_t v) {
    v &= 0x1fffff;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }

// Exclusive prefix sum over n items by one CTA of kScanThreads threads: rd(i)
// gives item i, wr(i, s) receives the sum of items before i.  Returns the total.
template <class Rd, class Wr>
__device__ int64_t cta_exclusive_scan(int n, Rd rd, Wr wr) {
    __shared__ int64_t warp_tot[kScanThreads / 32];
    __shared__ int64_t total_s;
    const int t = threadIdx.x;
    const int chunk = (n + kScanThreads - 1) / kScanThreads;
    const int b = min(n, t * chunk), e = min(n, b + chunk);
    int64_t sum = 0;
    for (int i = b; i < e; ++i) sum += rd(i);
    int64_t v = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if ((t & 31) >= o) v += u;
    }
    if ((t & 31) == 31) warp_tot[t >> 5] = v;
    __syncthreads();
    if (t < 32) {
        int64_t w = warp_tot[t];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t u = __shfl_up_sync(0xffffffffu, w, o);
            if (t >= o) w += u;
        }
        warp_tot[t] = w;
        if (t == 31) total_s = w;
    }
    __syncthreads();
    int64_t run = v - sum + ((t >> 5) ? warp_tot[(t >> 5) - 1] : 0);
    for (int i = b; i < e; ++i) {
        const int64_t x = rd(i);
        wr(i, run);
        run += x;
    }
    const int64_t tot = total_s;
    __syncthreads();
    return tot;
}

// ---------------------------------------------------------------- root cell and keys

__global__ __launch_bounds__(256) void bbox_partial_kernel(const double* __restrict__ pos, int64_t n,
                                                           double* __restrict__ part) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = gtid(); i < n; i += gstride())
        for (int d = 0; d < 3; ++d) {
            const double x = pos[3 * i + d];
            lo[d] = dmin(lo[d], x);
            hi[d] = dmax(hi[d], x);
        }
    __shared__ double s[6][256];
    for (int d = 0; d < 3; ++d) {
        s[d][threadIdx.x] = lo[d];
        s[3 + d][threadIdx.x] = hi[d];
    }
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
            for (int d = 0; d < 3; ++d) {
                s[d][threadIdx.x] = dmin(s[d][threadIdx.x], s[d][threadIdx.x + w]);
                s[3 + d][threadIdx.x] = dmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + w]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 6; ++d) part[6 * blockIdx.x + d] = s[d][0];
}

// Root cube as the host builder forms it; resets the build's header.
__global__ __launch_bounds__(256) void bbox_final_kernel(const double* __restrict__ part, int nb, int64_t n,
                                                          TreeHdr* h, TCell* cells) {
    __shared__ double s[6][256];
    {
        double l[3] = {1e300, 1e300, 1e300}, u[3] = {-1e300, -1e300, -1e300};
        for (int b = threadIdx.x; b < nb; b += 256)
            for (int d = 0; d < 3; ++d) {
                l[d] = dmin(l[d], part[6 * b + d]);
                u[d] = dmax(u[d], part[6 * b + 3 + d]);
            }
        for (int d = 0; d < 3; ++d) {
            s[d][threadIdx.x] = l[d];
            s[3 + d][threadIdx.x] = u[d];
        }
        __syncthreads();
        for (int w = 128; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w)
                for (int d = 0; d < 3; ++d) {
                    s[d][threadIdx.x] = dmin(s[d][threadIdx.x], s[d][threadIdx.x + w]);
                    s[3 + d][threadIdx.x] = dmax(s[3 + d][threadIdx.x], s[3 + d][threadIdx.x + w]);
                }
            __syncthreads();
        }
    }
    if (threadIdx.x != 0) return;
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
        lo[d] = s[d][0];
        hi[d] = s[3 + d][0];
    }
    double half = 0.0, cen[3];
    for (int d = 0; d < 3; ++d) {
        cen[d] = 0.5 * (lo[d] + hi[d]);
        half = dmax(half, 0.5 * (hi[d] - lo[d]));
    }
    half = half * 1.0001 + 1e-12;
    for (int d = 0; d < 3; ++d) h->root_lo[d] = cen[d] - half;
    h->half = half;
    h->scale = double(1 << kMaxLevel) / (2.0 * half);
    h->side0 = 2.0 * half;
    double xm = 0.0;
    for (int d = 0; d < 3; ++d) xm = dmax(xm, dmax(fabs(h->root_lo[d]), fabs(h->root_lo[d] + h->side0)));
    h->xmax = __double2float_ru(xm);
    for (int L = 0; L < kLevels + 2; ++L) h->level_begin[L] = L == 0 ? 0 : 1;
    h->n_groups = 0;
    h->n_fronts = 0;
    h->n_walk = 0;
    h->err = 0;
    h->n_epj_entries = h->n_spj_entries = 0;
    h->n_epep = h->n_epsp = 0;
    TCell& r = cells[0];
    r.begin = 0;
    r.end = (int32_t)n;
    r.level = 0;
    r.parent = -1;
    r.first_child = 0;
    r.n_child = 0;
    r.leaf = 0;
}

__global__ __launch_bounds__(256) void keys_kernel(const double* __restrict__ pos, int64_t n, const TreeHdr* h,
                                                   uint64_t* __restrict__ key, int32_t* __restrict__ val) {
    const double lo0 = h->root_lo[0], lo1 = h->root_lo[1], lo2 = h->root_lo[2], scale = h->scale;
    for (int64_t i = gtid(); i < n; i += gstride()) {
        const double lo[3] = {lo0, lo1, lo2};
        uint64_t k = 0;
        for (int d = 0; d < 3; ++d) {
            const double f = (pos[3 * i + d] - lo[d]) * scale;
            int64_t c = (int64_t)f;
            if (c < 0) c = 0;
            if (c > (1 << kMaxLevel) - 1) c = (1 << kMaxLevel) - 1;
            k |= spread3((uint64_t)c) << (2 - d);
        }
        key[i] = k;
        val[i] = (int32_t)i;
    }
}

// Sorted copies in the layouts the force kernels read.
__global__ __launch_bounds__(256) void gather_kernel(const int32_t* __restrict__ order, const double* __restrict__ pos,
                                                     const double* __restrict__ mass, const double* __restrict__ rs,
                                                     int64_t n, EpiDev* __restrict__ epi, EpjMix* __restrict__ epj,
                                                     double* __restrict__ m64, double* __restrict__ rs64,
                                                     EpjF32* __restrict__ epj32, int32_t* __restrict__ inv) {
    for (int64_t s = gtid(); s < n; s += gstride()) {
        const int64_t o = order[s];
        inv[o] = (int32_t)s;
        const double x = pos[3 * o], y = pos[3 * o + 1], z = pos[3 * o + 2];
        const double m = mass[o], r = rs[o];
        epi[s] = EpiDev{x, y, z, r};
        const EpjMix e{x, y, z, (float)m, (float)(r * r)};
        epj[s] = e;
        m64[s] = m;
        rs64[s] = r;
        EpjF32 f;
        f.xh = (float)x;
        f.yh = (float)y;
        f.zh = (float)z;
        f.xl = (float)(x - (double)f.xh);
        f.yl = (float)(y - (double)f.yh);
        f.zl = (float)(z - (double)f.zh);
        f.m = e.m;
        f.rs2 = e.rs2;
        epj32[s] = f;
    }
}

// ---------------------------------------------------------------- octree, level by level

// Octant boundaries of a cell at level L: child o holds [b[o], b[o + 1]).
__device__ __forceinline__ void octants(const uint64_t* __restrict__ skey, int begin, int end, int L, int b[9]) {
    const int shift = 3 * (kMaxLevel - 1 - L);
    b[0] = begin;
    b[8] = end;
    for (int o = 1; o < 8; ++o) {
        int lo = b[o - 1], hi = end;  // first index with digit >= o
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if ((int)((skey[mid] >> shift) & 7) < o) lo = mid + 1;
            else hi = mid;
        }
        b[o] = lo;
    }
}

// The cells of a level are split into kLevelBlocks contiguous chunks, one
// per CTA, so that the child numbering (children of a level in their parents'
// order) is a two-level scan: CTA sums here, their scan by one CTA, and the
// CTA-local scans when the children are written.
constexpr int kLevelBlocks = 1024;

__device__ __forceinline__ void level_chunk(const TreeHdr* h, int L, int& c0, int& c1) {
    const int lb = h->level_begin[L], le = h->level_begin[L + 1];
    const int per = (le - lb + kLevelBlocks - 1) / kLevelBlocks;
    c0 = min(le, lb + (int)blockIdx.x * per);
    c1 = min(le, c0 + per);
}

// Exclusive scan of one value per thread over a 256-thread CTA; *total gets
// the sum.  Every thread of the CTA must call it.
__device__ __forceinline__ int cta256_excl_scan(int v, int* total) {
    __shared__ int ws[8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int u = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += u;
    }
    if (lane == 31) ws[w] = x;
    __syncthreads();
    int base = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        base += k < w ? ws[k] : 0;
        tot += ws[k];
    }
    __syncthreads();
    *total = tot;
    return base + x - v;
}

__global__ __launch_bounds__(256) void split_kernel(TreeHdr* h, TCell* cells, int32_t* nch, int4* bnd,
                                                    int32_t* blocksum, const uint64_t* __restrict__ skey, int L,
                                                    int n_leaf) {
    if (h->err) return;
    int c0, c1;
    level_chunk(h, L, c0, c1);
    const int lb = h->level_begin[L];
    int sum = 0;
    if (c1 - c0 <= (int)(blockDim.x >> 5)) {
        // Few, large cells (the upper levels): a warp per cell, its seven
        // binary searches run by seven lanes at once instead of one after
        // another (each is a chain of dependent key loads).
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        if (c0 + w < c1) {
            const int c = c0 + w;
            TCell& cc = cells[c];
            const int cnt = cc.end - cc.begin;
            const bool leaf = cnt <= n_leaf || L >= kMaxLevel;
            int bo = cc.end;
            if (!leaf && lane < 7) {
                const int shift = 3 * (kMaxLevel - 1 - L);
                int lo = cc.begin, hi = cc.end;  // first index with digit >= lane + 1
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if ((int)((skey[mid] >> shift) & 7) < lane + 1) lo = mid + 1;
                    else hi = mid;
                }
                bo = lo;
            }
            int b[9];
            b[0] = cc.begin;
            b[8] = cc.end;
#pragma unroll
            for (int o = 1; o < 8; ++o) b[o] = __shfl_sync(0xffffffffu, bo, o - 1);
            if (lane == 0) {
                int k = 0;
                if (!leaf) {
                    for (int o = 0; o < 8; ++o) k += b[o + 1] > b[o];
                    bnd[2 * (c - lb)] = make_int4(b[1], b[2], b[3], b[4]);
                    bnd[2 * (c - lb) + 1] = make_int4(b[5], b[6], b[7], b[8]);
                }
                cc.leaf = leaf;
                cc.n_child = k;
                nch[c - lb] = k;
                sum = k;
            }
        }
    } else {
        for (int c = c0 + (int)threadIdx.x; c < c1; c += blockDim.x) {
            TCell& cc = cells[c];
            const int cnt = cc.end - cc.begin;
            const bool leaf = cnt <= n_leaf || L >= kMaxLevel;
            int k = 0;
            if (!leaf) {
                int b[9];
                octants(skey, cc.begin, cc.end, L, b);
                for (int o = 0; o < 8; ++o) k += b[o + 1] > b[o];
                // The octant ends, for the fill of this level.
                bnd[2 * (c - lb)] = make_int4(b[1], b[2], b[3], b[4]);
                bnd[2 * (c - lb) + 1] = make_int4(b[5], b[6], b[7], b[8]);
            }
            cc.leaf = leaf;
            cc.n_child = k;
            nch[c - lb] = k;
            sum += k;
        }
    }
    int tot;
    (void)cta256_excl_scan(sum, &tot);
    if (threadIdx.x == 0) blocksum[blockIdx.x] = tot;
}

__global__ __launch_bounds__(kScanThreads) void level_scan_kernel(TreeHdr* h, int32_t* blocksum, int L, int cap) {
    if (h->err) return;
    const int le = h->level_begin[L + 1];
    const int64_t tot = cta_exclusive_scan(
        kLevelBlocks, [&](int i) { return (int64_t)blocksum[i]; },
        [&](int i, int64_t v) { blocksum[i] = (int32_t)min(v, (int64_t)cap); });
    if (threadIdx.x == 0) {
        if ((int64_t)le + tot > cap) {
            h->err |= kErrCells;
            h->level_begin[L + 2] = le;
        } else {
            h->level_begin[L + 2] = le + (int)tot;
        }
    }
}

__global__ __launch_bounds__(256) void fill_kernel(TreeHdr* h, TCell* cells, const int32_t* __restrict__ nch,
                                                   const int4* __restrict__ bnd, const int32_t* __restrict__ blockoff,
                                                   int L) {
    if (h->err) return;
    int c0, c1;
    level_chunk(h, L, c0, c1);
    const int lb = h->level_begin[L], le = h->level_begin[L + 1];
    int run = le + blockoff[blockIdx.x];
    for (int t0 = c0; t0 < c1; t0 += blockDim.x) {  // uniform trip count over the CTA
        const int c = t0 + (int)threadIdx.x;
        const int k_c = c < c1 ? nch[c - lb] : 0;
        int tot;
        const int off = cta256_excl_scan(k_c, &tot);
        if (c < c1 && k_c > 0) {
            TCell& cc = cells[c];
            const int first = run + off;
            cc.first_child = first;
            const int4 u = bnd[2 * (c - lb)], v = bnd[2 * (c - lb) + 1];
            const int b[9] = {cc.begin, u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w};
            int k = 0;
            for (int o = 0; o < 8; ++o) {
                if (b[o + 1] <= b[o]) continue;
                TCell& ch = cells[first + k++];
                ch.begin = b[o];
                ch.end = b[o + 1];
                ch.level = L + 1;
                ch.parent = c;
                ch.first_child = 0;
                ch.n_child = 0;
                ch.leaf = 0;
            }
        } else if (c < c1) {
            cells[c].first_child = run + off;
        }
        run += tot;
    }
}

// Moments, boxes and the SPJ records: LEAVES, every leaf of the tree from
// its particles; otherwise the inner cells of level L from their children
// (run deepest level first).
// The cells in moments classes, so that the threads of a warp run loops of
// the same length (GB300 issues each FP64 instruction for the whole warp,
// whatever its active lanes): leaves by particle count, largest first, then
// the inner cells of each level by child count, most first.
__device__ __forceinline__ int cell_bin(const TCell& c) {
    if (c.leaf) {
        const int n = c.end - c.begin;
        return kLeafBins - 1 - (n < kLeafBins - 1 ? n : kLeafBins - 1);
    }
    return kLeafBins + 8 * c.level + (8 - c.n_child);
}

// First slot of class b in the cell list (after the scatter).
__device__ __forceinline__ int bin_start(const TreeHdr* h, int b) { return b == 0 ? 0 : h->cell_cursor[b - 1]; }

__global__ __launch_bounds__(256) void cell_hist_kernel(TreeHdr* h, const TCell* __restrict__ cells) {
    __shared__ int hs[kCellBins];
    for (int b = threadIdx.x; b < kCellBins; b += blockDim.x) hs[b] = 0;
    __syncthreads();
    if (!h->err) {
        const int nc = h->level_begin[kLevels];
        for (int64_t c = gtid(); c < nc; c += gstride()) atomicAdd(&hs[cell_bin(cells[c])], 1);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kCellBins; b += blockDim.x)
        if (hs[b]) atomicAdd(&h->cell_hist[b], hs[b]);
}

__global__ void cell_scan_kernel(TreeHdr* h) {
    if (threadIdx.x != 0) return;
    int run = 0;
    for (int b = 0; b < kCellBins; ++b) {
        h->cell_cursor[b] = run;
        run += h->cell_hist[b];
    }
}

__global__ __launch_bounds__(256) void cell_scatter_kernel(TreeHdr* h, const TCell* __restrict__ cells,
                                                           int32_t* __restrict__ order) {
    __shared__ int hs[kCellBins], base[kCellBins];
    const int nc = h->err ? 0 : h->level_begin[kLevels];
    for (int64_t c0 = (int64_t)blockIdx.x * blockDim.x; c0 < nc; c0 += gstride()) {
        for (int b = threadIdx.x; b < kCellBins; b += blockDim.x) hs[b] = 0;
        __syncthreads();
        const int64_t c = c0 + threadIdx.x;
        int b = -1, r = 0;
        if (c < nc) {
            b = cell_bin(cells[c]);
            r = atomicAdd(&hs[b], 1);
        }
        __syncthreads();
        for (int k = threadIdx.x; k < kCellBins; k += blockDim.x)
            base[k] = hs[k] ? atomicAdd(&h->cell_cursor[k], hs[k]) : 0;
        __syncthreads();
        if (b >= 0) order[base[b] + r] = (int32_t)c;
        __syncthreads();
    }
}

template <bool LEAVES>
__global__ __launch_bounds__(256) void moments_kernel(const TreeHdr* h, TCell* cells, TCellW* cw, CMom* mom,
                                                      const EpiDev* __restrict__ epi, const double* __restrict__ m64,
                                                      int L, double inv_theta2, SpjMix* spj, SpjF32* spj32,
                                                      SpjQ64* spjq, const int32_t* __restrict__ order) {
    if (h->err) return;
    const int lb = LEAVES ? 0 : bin_start(h, kLeafBins + 8 * L);
    const int le = LEAVES ? bin_start(h, kLeafBins) : bin_start(h, kLeafBins + 8 * L + 8);
    for (int64_t t = lb + gtid(); t < le; t += gstride()) {
        const int64_t c = order[t];
        TCell& cc = cells[c];
        const double side = ldexp(h->side0, -cc.level);
        double m = 0, mx[3] = {0, 0, 0}, q[6] = {0, 0, 0, 0, 0, 0};
        double ilo[3], ihi[3], olo[3], ohi[3];
        for (int d = 0; d < 3; ++d) {
            ilo[d] = olo[d] = 1e300;
            ihi[d] = ohi[d] = -1e300;
        }
        double rsm = 0.0;
        if (cc.leaf) {
            for (int i = cc.begin; i < cc.end; ++i) {
                const EpiDev e = epi[i];
                const double mi = m64[i];
                const double x[3] = {e.x, e.y, e.z};
                m += mi;
                for (int d = 0; d < 3; ++d) {
                    mx[d] += mi * x[d];
                    ilo[d] = kmin(ilo[d], x[d]);
                    ihi[d] = kmax(ihi[d], x[d]);
                    olo[d] = kmin(olo[d], x[d] - e.rs);
                    ohi[d] = kmax(ohi[d], x[d] + e.rs);
                }
                rsm = kmax(rsm, e.rs);
            }
        } else {
            for (int k = 0; k < cc.n_child; ++k) {
                const int ci = cc.first_child + k;
                const CMom& cm = mom[ci];
                const TCell& ch = cells[ci];
                m += cm.m;
                for (int d = 0; d < 3; ++d) {
                    mx[d] += cm.mx[d];
                    ilo[d] = kmin(ilo[d], ch.in_lo[d]);
                    ihi[d] = kmax(ihi[d], ch.in_hi[d]);
                    olo[d] = kmin(olo[d], ch.out_lo[d]);
                    ohi[d] = kmax(ohi[d], ch.out_hi[d]);
                }
                rsm = kmax(rsm, (double)ch.rs_max);
            }
        }
        double com[3];
        for (int d = 0; d < 3; ++d) com[d] = m > 0 ? mx[d] / m : 0.5 * (ilo[d] + ihi[d]);
        if (cc.leaf) {
            for (int i = cc.begin; i < cc.end; ++i) {
                const EpiDev e = epi[i];
                const double mi = m64[i];
                const double dx = e.x - com[0], dy = e.y - com[1], dz = e.z - com[2];
                q[0] += mi * dx * dx;
                q[1] += mi * dy * dy;
                q[2] += mi * dz * dz;
                q[3] += mi * dx * dy;
                q[4] += mi * dx * dz;
                q[5] += mi * dy * dz;
            }
        } else {
            for (int k = 0; k < cc.n_child; ++k) {
                const int ci = cc.first_child + k;
                const CMom& cm = mom[ci];
                const TCell& ch = cells[ci];
                const double dx = ch.com[0] - com[0], dy = ch.com[1] - com[1], dz = ch.com[2] - com[2];
                q[0] += cm.q[0] + cm.m * dx * dx;
                q[1] += cm.q[1] + cm.m * dy * dy;
                q[2] += cm.q[2] + cm.m * dz * dz;
                q[3] += cm.q[3] + cm.m * dx * dy;
                q[4] += cm.q[4] + cm.m * dx * dz;
                q[5] += cm.q[5] + cm.m * dy * dz;
            }
        }
        for (int d = 0; d < 3; ++d) {
            cc.com[d] = com[d];
            cc.in_lo[d] = ilo[d];
            cc.in_hi[d] = ihi[d];
            cc.out_lo[d] = olo[d];
            cc.out_hi[d] = ohi[d];
        }
        cc.crit = side * side * inv_theta2;
        cc.rs_max = __double2float_ru(rsm);
        TCellW w;
        for (int d = 0; d < 3; ++d) {
            w.com[d] = (float)com[d];
            w.in_lo[d] = (float)ilo[d];
            w.in_hi[d] = (float)ihi[d];
            w.out_lo[d] = (float)olo[d];
            w.out_hi[d] = (float)ohi[d];
        }
        w.crit = (float)cc.crit;
        w.begin = cc.begin;
        w.end = cc.end;
        w.first_child = cc.first_child;
        w.n_child = cc.n_child;
        w.leaf = cc.leaf;
        w.parent = cc.parent;
        w.level = cc.level;
        w.pad1 = 0;
        cw[c] = w;
        CMom& o = mom[c];
        o.m = m;
        for (int d = 0; d < 3; ++d) o.mx[d] = mx[d];
        for (int k = 0; k < 6; ++k) o.q[k] = q[k];
        // SPJ records of the cell, as the dispatch path packs them.
        const double tr = q[0] + q[1] + q[2];
        SpjMix s;
        s.x = com[0];
        s.y = com[1];
        s.z = com[2];
        s.m = (float)m;
        s.pad0 = 0.f;
        s.Q[0] = (float)(3.0 * q[0] - tr);
        s.Q[1] = (float)(3.0 * q[1] - tr);
        s.Q[2] = (float)(3.0 * q[2] - tr);
        s.Q[3] = (float)(3.0 * q[3]);
        s.Q[4] = (float)(3.0 * q[4]);
        s.Q[5] = (float)(3.0 * q[5]);
        s.tr = (float)tr;
        s.pad1 = 0.f;
        spj[c] = s;
        SpjF32 f;
        f.xh = (float)com[0];
        f.yh = (float)com[1];
        f.zh = (float)com[2];
        f.xl = (float)(com[0] - (double)f.xh);
        f.yl = (float)(com[1] - (double)f.yh);
        f.zl = (float)(com[2] - (double)f.zh);
        f.m = s.m;
        f.tr = s.tr;
        for (int k = 0; k < 6; ++k) f.Q[k] = s.Q[k];
        f.pad[0] = f.pad[1] = 0.f;
        spj32[c] = f;
        SpjQ64 d64;
        d64.m = m;
        for (int k = 0; k < 6; ++k) d64.q[k] = q[k];
        d64.pad = 0.0;
        spjq[c] = d64;
    }
}

// ---------------------------------------------------------------- groups and walks

__device__ __forceinline__ bool group_eligible(const TCell& c, int n_group) {
    return c.end - c.begin <= n_group || c.leaf;
}

__global__ __launch_bounds__(256) void group_mark_kernel(const TreeHdr* h, const TCell* __restrict__ cells,
                                                         int32_t* __restrict__ group_at, int n_group) {
    if (h->err) return;
    const int nc = h->level_begin[kLevels];
    for (int64_t c = gtid(); c < nc; c += gstride()) {
        const TCell& cc = cells[c];
        if (!group_eligible(cc, n_group)) continue;
        if (c > 0 && group_eligible(cells[cc.parent], n_group)) continue;
        group_at[cc.begin] = (int32_t)c;
    }
}

struct NonNegative {
    __host__ __device__ __forceinline__ bool operator()(const int32_t& v) const { return v >= 0; }
};

__device__ __forceinline__ double box_dist2_point(const double lo[3], const double hi[3], const double p[3]) {
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        double dd = 0.0;
        if (p[d] < lo[d]) dd = lo[d] - p[d];
        else if (p[d] > hi[d]) dd = p[d] - hi[d];
        s += dd * dd;
    }
    return s;
}

__device__ __forceinline__ bool box_overlap(const double alo[3], const double ahi[3], const double blo[3],
                                            const double bhi[3]) {
    for (int d = 0; d < 3; ++d)
        if (alo[d] > bhi[d] || blo[d] > ahi[d]) return false;
    return true;
}

__device__ __forceinline__ bool exact_open(const TCell& gc, const TCell& cc) {
    const double com[3] = {cc.com[0], cc.com[1], cc.com[2]};
    const double r2 = box_dist2_point(gc.in_lo, gc.in_hi, com);
    return r2 <= cc.crit || box_overlap(gc.out_lo, gc.out_hi, cc.in_lo, cc.in_hi) ||
           box_overlap(gc.in_lo, gc.in_hi, cc.out_lo, cc.out_hi);
}

// box_overlap on rounded boxes: 1 overlap, 0 none, 2 unknown.  Rounding to
// nearest is monotonic, so a strict inequality between rounded values holds
// for the FP64 values too: one rounded a > b separates the boxes, and strict
// a < b on every pair proves the overlap; only ties are left to FP64.
__device__ __forceinline__ int overlap3(const float alo[3], const float ahi[3], const float blo[3], const float bhi[3]) {
    const bool sep = (alo[0] > bhi[0]) | (blo[0] > ahi[0]) | (alo[1] > bhi[1]) | (blo[1] > ahi[1]) |
                     (alo[2] > bhi[2]) | (blo[2] > ahi[2]);
    if (sep) return 0;
    const bool ovl = (alo[0] < bhi[0]) & (blo[0] < ahi[0]) & (alo[1] < bhi[1]) & (blo[1] < ahi[1]) &
                     (alo[2] < bhi[2]) & (blo[2] < ahi[2]);
    return ovl ? 1 : 2;
}

// r2 <= crit of the FP64 test from rounded data: 1 open, 0 not, 2 unknown.
// Every coordinate is below X in magnitude, so each rounded input is off by
// at most u X and each per-axis distance dd by at most E = 3 u X + u S, with
// S the sum of the three rounded distances; the sum of squares then differs
// from the FP64 one by at most E (2 S + 3 E) plus 3 u r2 of its own rounding
// (the bound is doubled to cover the rounding of the bound itself).
__device__ __forceinline__ int dist3(const float glo[3], const float ghi[3], const TCellW& w, float X) {
    float r2 = 0.f, S = 0.f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float dd = fmaxf(fmaxf(glo[d] - w.com[d], w.com[d] - ghi[d]), 0.f);
        r2 += dd * dd;
        S += dd;
    }
    const float E = 3.f * kU * X + kU * S;
    const float B = 2.f * (E * (2.f * S + 3.f * E) + 3.f * kU * r2);
    if (r2 + B < w.crit * (1.f - 2.f * kU)) return 1;
    if (r2 - B > w.crit * (1.f + 2.f * kU)) return 0;
    return 2;
}

struct WalkCtx {
    const TCellW* __restrict__ cw;
    const TCell* __restrict__ cells;
    int gcell;
    float in_lo[3], in_hi[3], out_lo[3], out_hi[3];
    float X;
    bool open_all;
};

__device__ __forceinline__ void load_ctx(WalkCtx& x, const TCellW* cw, const TCell* cells, int gcell, float X,
                                         bool open_all) {
    x.cw = cw;
    x.cells = cells;
    x.gcell = gcell;
    const TCellW g = cw[gcell];
    for (int d = 0; d < 3; ++d) {
        x.in_lo[d] = g.in_lo[d];
        x.in_hi[d] = g.in_hi[d];
        x.out_lo[d] = g.out_lo[d];
        x.out_hi[d] = g.out_hi[d];
    }
    x.X = X;
    x.open_all = open_all;
}

// The FP64 opening test of the host builder, decided in FP32 where possible.
__device__ __forceinline__ bool open_cell(const WalkCtx& x, int c, const TCellW& w) {
    if (x.open_all) return true;
    const int d = dist3(x.in_lo, x.in_hi, w, x.X);
    if (d == 1) return true;
    const int o1 = overlap3(x.out_lo, x.out_hi, w.in_lo, w.in_hi);
    if (o1 == 1) return true;
    const int o2 = overlap3(x.in_lo, x.in_hi, w.out_lo, w.out_hi);
    if (o2 == 1) return true;
    if (d == 0 && o1 == 0 && o2 == 0) return false;
    return exact_open(x.cells[x.gcell], x.cells[c]);
}

// Lists of frontier cell f's subtree for the group of x, appended at ne / ns:
// counts (FILL false) or writes (FILL true) the entries in the host builder's
// depth-first order.
template <bool FILL>
__device__ void walk_subtree(const WalkCtx& x, int f, const TCellW& fw, int& ne, int& ns, int32_t* __restrict__ oe,
                             int32_t* __restrict__ os) {
    // f itself, then depth-first below it.  Expanding an opened cell decides
    // all its children at once (independent loads); closed cells and leaves
    // are listed at once while no opened inner child precedes them, the walk
    // descends into the first opened inner child, and the later siblings wait
    // on the stack with their decision (2 low bits: 0 closed, 1 leaf, 2 inner).
    if (!open_cell(x, f, fw)) {
        if (FILL) os[ns] = f;
        ++ns;
        return;
    }
    if (fw.leaf) {
        if (FILL)
            for (int i = fw.begin; i < fw.end; ++i) oe[ne + (i - fw.begin)] = i;
        ne += fw.end - fw.begin;
        return;
    }
    uint32_t stack[kStack];
    int sp = 0;
    int fc = fw.first_child, nc = fw.n_child;
    for (;;) {
        uint32_t dec = 0;
        int next = -1, next_fc = 0, next_nc = 0;
        for (int k = 0; k < nc; ++k) {
            const int c = fc + k;
            const TCellW w = x.cw[c];
            const int code = !open_cell(x, c, w) ? 0 : (w.leaf ? 1 : 2);
            if (next < 0) {
                if (code == 0) {
                    if (FILL) os[ns] = c;
                    ++ns;
                } else if (code == 1) {
                    if (FILL)
                        for (int i = w.begin; i < w.end; ++i) oe[ne + (i - w.begin)] = i;
                    ne += w.end - w.begin;
                } else {
                    next = k;
                    next_fc = w.first_child;
                    next_nc = w.n_child;
                }
            } else {
                dec |= (uint32_t)code << (2 * k);
            }
        }
        if (next >= 0) {
            for (int k = nc - 1; k > next; --k) stack[sp++] = ((uint32_t)(fc + k) << 2) | ((dec >> (2 * k)) & 3u);
            fc = next_fc;
            nc = next_nc;
            continue;
        }
        for (;;) {
            if (sp == 0) return;
            const uint32_t e = stack[--sp];
            const int c = (int)(e >> 2);
            const uint32_t code = e & 3u;
            if (code == 0) {
                if (FILL) os[ns] = c;
                ++ns;
            } else if (code == 1) {
                const int b0 = x.cw[c].begin, b1 = x.cw[c].end;
                if (FILL)
                    for (int i = b0; i < b1; ++i) oe[ne + (i - b0)] = i;
                ne += b1 - b0;
            } else {
                fc = x.cw[c].first_child;
                nc = x.cw[c].n_child;
                break;
            }
        }
    }
}

// Frontier cells f0 .. f1-1 (consecutive in frontier order) for one group.
// A frontier cell is walked if the group opens all its ancestors; a closed
// ancestor ends it and is listed by the frontier cell that starts its range.
// The decisions along the current ancestor chain are kept by level, so a
// frontier cell climbs its parent links only up to the deepest ancestor it
// shares with the previous one (cells are in Morton order, so an ancestor of
// two frontier cells is an ancestor of every frontier cell between them) and
// tests only the ancestors below it.
template <bool FILL>
__device__ void walk_chunk(const WalkCtx& x, const int32_t* __restrict__ fronts, int f0, int f1, int& ne, int& ns,
                           int32_t* __restrict__ oe, int32_t* __restrict__ os) {
    ne = ns = 0;
    int cache_c[kLevels];        // ancestor of the current chain at each level, all tested
    int n_cached = 0;            // levels [0, n_cached) are valid
    int first_closed = kLevels;  // the closed one among them (only the last can be)
    for (int fi = f0; fi < f1; ++fi) {
        const int f = fronts[fi];
        const TCellW fw = x.cw[f];
        // Climb to the deepest cached ancestor; the others are new.
        int fresh[kLevels];  // new ancestors, deepest first
        int nf = 0;
        int c = fw.parent, lvl = fw.level - 1;
        while (c >= 0 && !(lvl < n_cached && cache_c[lvl] == c)) {
            fresh[nf++] = c;
            c = x.cw[c].parent;
            --lvl;
        }
        n_cached = lvl + 1;
        if (first_closed >= n_cached) first_closed = kLevels;
        int closed_at = -1;
        if (first_closed < kLevels) {
            closed_at = cache_c[first_closed];
        } else {
            for (int k = nf - 1; k >= 0; --k) {  // root side first
                const int a = fresh[k];
                const bool op = open_cell(x, a, x.cw[a]);
                cache_c[n_cached++] = a;
                if (!op) {
                    first_closed = n_cached - 1;
                    closed_at = a;
                    break;
                }
            }
        }
        if (closed_at >= 0) {
            if (fw.begin == x.cw[closed_at].begin) {
                if (FILL) os[ns] = closed_at;
                ++ns;
            }
            continue;
        }
        walk_subtree<FILL>(x, f, fw, ne, ns, oe, os);
    }
}

__device__ __forceinline__ int cost_bucket(float cost) {
    if (!(cost > 1.f)) return 0;
    const int b = (int)(log2f(cost) * 8.f);
    return b < kBuckets ? b : kBuckets - 1;
}

constexpr int kChunk = 2;  // frontier cells per task

__device__ __forceinline__ int64_t n_chunks(const TreeHdr* h) { return (h->n_fronts + kChunk - 1) / kChunk; }

__global__ void task_check_kernel(TreeHdr* h, int64_t cap_tasks) {
    if (threadIdx.x != 0) return;
    h->walk_cursor[0] = h->walk_cursor[1] = 0;
    if (h->err) return;
    if ((int64_t)h->n_groups * n_chunks(h) > cap_tasks) h->err |= kErrTasks;
}

// The walk passes take tasks a warp at a time from a counter: task costs
// differ by orders of magnitude (a chunk next to the group against one whose
// ancestors the group closes), so a static split leaves SMs idle at the end.
// Lane l of a warp takes task base + l, so a warp walks one chunk for 32
// neighbouring groups.
__device__ __forceinline__ int64_t next_tasks(unsigned long long* cursor) {
    unsigned long long base = 0;
    if ((threadIdx.x & 31) == 0) base = atomicAdd(cursor, 32ull);
    return (int64_t)__shfl_sync(0xffffffffu, base, 0);
}

// Task t = (chunk q = t / n_groups, group g = t % n_groups) walks frontier
// cells kChunk q .. kChunk q + kChunk - 1 for group g: the threads of a warp
// walk the same subtrees for neighbouring groups.  Counts are stored at t.
__global__ __launch_bounds__(128) void walk_task_count_kernel(TreeHdr* h, const TCellW* __restrict__ cw,
                                                              const TCell* __restrict__ cells,
                                                              const int32_t* __restrict__ groups,
                                                              const int32_t* __restrict__ fronts, int32_t* task_e,
                                                              int32_t* task_s, bool open_all) {
    if (h->err) return;
    const int64_t ng = h->n_groups, nf = h->n_fronts, T = ng * n_chunks(h);
    const float X = h->xmax;
    for (;;) {
        const int64_t t = next_tasks(&h->walk_cursor[0]) + (threadIdx.x & 31);
        if (t - (threadIdx.x & 31) >= T) break;
        if (t >= T) continue;
        const int q = (int)(t / ng), g = (int)(t - (int64_t)q * ng);
        WalkCtx x;
        load_ctx(x, cw, cells, groups[g], X, open_all);
        int ne, ns;
        walk_chunk<false>(x, fronts, q * kChunk, (int)min(nf, (int64_t)(q + 1) * kChunk), ne, ns, nullptr,
                          nullptr);
        task_e[t] = ne;
        task_s[t] = ns;
    }
}

// Per group: offsets of its tasks within its lists (in frontier order), the
// list lengths, the walk descriptor and the work-queue bucket.
__global__ __launch_bounds__(128) void group_reduce_kernel(TreeHdr* h, const TCell* __restrict__ cells,
                                                           const int32_t* __restrict__ groups, WalkDesc* walks,
                                                           int32_t* task_e, int32_t* task_s, int32_t* cnt_e,
                                                           int32_t* cnt_s, int32_t* bucket, double rcut2) {
    if (h->err) return;
    const int64_t ng = h->n_groups, nq = n_chunks(h);
    for (int64_t g = gtid(); g < ng; g += gstride()) {
        // Counts are read kB chunks at a time before their offsets are
        // written back: loads that follow a store to the same array would
        // otherwise wait one memory latency per chunk.
        constexpr int kB = 32;
        int64_t re = 0, rs = 0;
        for (int64_t q0 = 0; q0 < nq; q0 += kB) {
            int e[kB], s[kB];
#pragma unroll
            for (int k = 0; k < kB; ++k) {
                const int64_t t = (q0 + k) * ng + g;
                e[k] = q0 + k < nq ? task_e[t] : 0;
                s[k] = q0 + k < nq ? task_s[t] : 0;
            }
#pragma unroll
            for (int k = 0; k < kB; ++k) {
                if (q0 + k < nq) {
                    const int64_t t = (q0 + k) * ng + g;
                    task_e[t] = (int32_t)re;
                    task_s[t] = (int32_t)rs;
                }
                re += e[k];
                rs += s[k];
            }
        }
        const int ne = (int)re, ns = (int)rs;
        const TCell& gc = cells[groups[g]];
        WalkDesc d;
        d.epj_begin = 0;
        d.spj_begin = 0;
        d.i_begin = gc.begin;
        d.n_i = gc.end - gc.begin;
        d.n_epj = ne;
        d.n_spj = ns;
        d.cx = 0.5 * (gc.in_lo[0] + gc.in_hi[0]);
        d.cy = 0.5 * (gc.in_lo[1] + gc.in_hi[1]);
        d.cz = 0.5 * (gc.in_lo[2] + gc.in_hi[2]);
        d.hx = __double2float_ru(dmax(gc.in_hi[0] - d.cx, d.cx - gc.in_lo[0]));
        d.hy = __double2float_ru(dmax(gc.in_hi[1] - d.cy, d.cy - gc.in_lo[1]));
        d.hz = __double2float_ru(dmax(gc.in_hi[2] - d.cz, d.cz - gc.in_lo[2]));
        d.rs_max = gc.rs_max;
        d.rcut2 = rcut2;
        d.part = 0;
        d.pad[0] = d.pad[1] = d.pad[2] = 0.f;
        walks[g] = d;
        cnt_e[g] = ne;
        cnt_s[g] = ns;
        const float cost = (float)d.n_i * ((float)ne + 2.f * (float)ns);
        const int b = cost_bucket(cost);
        bucket[g] = b;
        atomicAdd(&h->hist[b], 1);
        atomicAdd(&h->n_epep, (unsigned long long)d.n_i * (unsigned long long)ne);
        atomicAdd(&h->n_epsp, (unsigned long long)d.n_i * (unsigned long long)ns);
    }
}

__global__ __launch_bounds__(kScanThreads) void walk_scan_kernel(TreeHdr* h, WalkDesc* walks, const int32_t* cnt_e,
                                                                 const int32_t* cnt_s, int64_t cap_e, int64_t cap_s) {
    if (h->err) {
        if (threadIdx.x == 0) {
            h->n_walk = 0;
            h->err_sticky |= h->err;
        }
        return;
    }
    const int ng = h->n_groups;
    const int64_t te = cta_exclusive_scan(
        ng, [&](int i) { return (int64_t)cnt_e[i]; }, [&](int i, int64_t v) { walks[i].epj_begin = v; });
    const int64_t ts = cta_exclusive_scan(
        ng, [&](int i) { return (int64_t)cnt_s[i]; }, [&](int i, int64_t v) { walks[i].spj_begin = v; });
    if (threadIdx.x == 0) {
        h->n_epj_entries = te;
        h->n_spj_entries = ts;
        int32_t err = 0;
        if (te > cap_e) err |= kErrEpj;
        if (ts > cap_s) err |= kErrSpj;
        h->err = err;
        h->err_sticky |= err;
        h->n_walk = err ? 0 : ng;
        if (!err) {
            h->total_epep += h->n_epep;
            h->total_epsp += h->n_epsp;
        }
    }
}

__global__ __launch_bounds__(128) void walk_task_fill_kernel(TreeHdr* h, const TCellW* __restrict__ cw,
                                                             const TCell* __restrict__ cells,
                                                             const int32_t* __restrict__ groups,
                                                             const int32_t* __restrict__ fronts,
                                                             const WalkDesc* __restrict__ walks,
                                                             const int32_t* __restrict__ task_e,
                                                             const int32_t* __restrict__ task_s, int32_t* id_epj,
                                                             int32_t* id_spj, bool open_all) {
    if (h->err) return;
    const int64_t ng = h->n_groups, nf = h->n_fronts, T = ng * n_chunks(h);
    const float X = h->xmax;
    for (;;) {
        const int64_t t = next_tasks(&h->walk_cursor[1]) + (threadIdx.x & 31);
        if (t - (threadIdx.x & 31) >= T) break;
        if (t >= T) continue;
        const int q = (int)(t / ng), g = (int)(t - (int64_t)q * ng);
        WalkCtx x;
        load_ctx(x, cw, cells, groups[g], X, open_all);
        const WalkDesc& d = walks[g];
        int ne, ns;
        walk_chunk<true>(x, fronts, q * kChunk, (int)min(nf, (int64_t)(q + 1) * kChunk), ne, ns,
                         id_epj + d.epj_begin + task_e[t], id_spj + d.spj_begin + task_s[t]);
    }
}

// Work queue: walks by descending cost bucket (ties in no fixed order; the
// order changes which CTA runs a walk, not its results).
__global__ __launch_bounds__(256) void queue_scatter_kernel(TreeHdr* h, const int32_t* __restrict__ bucket,
                                                            int32_t* __restrict__ order) {
    __shared__ int32_t off[kBuckets];
    if (h->err) return;
    if (threadIdx.x == 0) {
        int run = 0;
        for (int b = kBuckets - 1; b >= 0; --b) {
            off[b] = run;
            run += h->hist[b];
        }
    }
    __syncthreads();
    const int ng = h->n_groups;
    for (int64_t g = gtid(); g < ng; g += gstride()) {
        const int b = bucket[g];
        order[off[b] + atomicAdd(&h->cursor[b], 1)] = (int32_t)g;
    }
}

// ---------------------------------------------------------------- integration

__global__ __launch_bounds__(256) void kick_drift_kernel(double* __restrict__ pos, double* __restrict__ vel,
                                                         const double* __restrict__ acc, int64_t n3, double dt_kick,
                                                         double dt_drift) {
    for (int64_t k = gtid(); k < n3; k += gstride()) {
        const double v = vel[k] + acc[k] * dt_kick;
        vel[k] = v;
        pos[k] = pos[k] + v * dt_drift;
    }
}

// Results back to particle order (the functor's retrieve), then the closing kick.
__global__ __launch_bounds__(256) void finish_kernel(const TreeHdr* h, const int32_t* __restrict__ order,
                                                     const Accp* __restrict__ accp, const int32_t* __restrict__ nnb,
                                                     int64_t n, double* __restrict__ acc, double* __restrict__ pot,
                                                     int32_t* __restrict__ n_ngb, double* __restrict__ vel,
                                                     double dt_kick) {
    if (h->n_walk == 0 && n > 0) return;  // failed build: keep the last forces
    for (int64_t s = gtid(); s < n; s += gstride()) {
        const int64_t o = order[s];
        const Accp a = accp[s];
        acc[3 * o] = a.x;
        acc[3 * o + 1] = a.y;
        acc[3 * o + 2] = a.z;
        pot[o] = a.w;
        n_ngb[o] = nnb[s];
        if (dt_kick != 0.0) {
            vel[3 * o] += a.x * dt_kick;
            vel[3 * o + 1] += a.y * dt_kick;
            vel[3 * o + 2] += a.z * dt_kick;
        }
    }
}

// Kinetic energy and the soft potential energy 1/2 sum m (pot + G m / r_out),
// the second term removing each particle's interaction with itself (the
// kernel counts the self pair as a cutoff pair, src/force_gpu_cuda.cu:62-76).
constexpr int kEnergyBlocks = 256;
__global__ __launch_bounds__(256) void energy_partial_kernel(const double* __restrict__ vel,
                                                             const double* __restrict__ mass,
                                                             const double* __restrict__ pot, int64_t n,
                                                             double self_coef, double* __restrict__ part) {
    double ek = 0.0, ep = 0.0;
    for (int64_t i = gtid(); i < n; i += gstride()) {
        const double m = mass[i];
        const double vx = vel[3 * i], vy = vel[3 * i + 1], vz = vel[3 * i + 2];
        ek += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        ep += 0.5 * m * (pot[i] + self_coef * m);
    }
    __shared__ double sk[256], sp[256];
    sk[threadIdx.x] = ek;
    sp[threadIdx.x] = ep;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            sk[threadIdx.x] += sk[threadIdx.x + w];
            sp[threadIdx.x] += sp[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = sk[0];
        part[2 * blockIdx.x + 1] = sp[0];
    }
}

__global__ void energy_final_kernel(const double* __restrict__ part, int nb, double* __restrict__ out) {
    if (threadIdx.x != 0) return;
    double ek = 0.0, ep = 0.0;
    for (int b = 0; b < nb; ++b) {
        ek += part[2 * b];
        ep += part[2 * b + 1];
    }
    out[0] = ek;
    out[1] = ep;
}

// ---------------------------------------------------------------- per-step sample

// One sampled particle at one step: the mixed-precision result and an FP64
// evaluation over the same lists (the plain FP64 kernel's pair formulas,
// summed over the lanes of a warp).
struct SampleRec {
    double acc[3], pot;
    double acc64[3], pot64;
    int32_t n_ngb, n_ngb64, step, pad;
};
static_assert(sizeof(SampleRec) == 80, "SampleRec layout");

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ __launch_bounds__(128) void sample_kernel(const TreeHdr* h, const int64_t* __restrict__ sample,
                                                     int n_sample, const int32_t* __restrict__ inv,
                                                     const WalkDesc* __restrict__ walks,
                                                     const EpiDev* __restrict__ epi, const EpjMix* __restrict__ epj,
                                                     const double* __restrict__ m64, const double* __restrict__ rs64,
                                                     const SpjMix* __restrict__ spj, const SpjQ64* __restrict__ spjq,
                                                     const int32_t* __restrict__ id_epj,
                                                     const int32_t* __restrict__ id_spj, double eps2, double G,
                                                     const Accp* __restrict__ accp, const int32_t* __restrict__ nnb,
                                                     SampleRec* hist, int hist_steps) {
    if (h->n_walk == 0) return;
    const int slot = h->sample_slot;
    if (slot < 0 || slot >= hist_steps) return;
    const int lane = threadIdx.x & 31;
    const int ng = h->n_walk;
    for (int64_t q = gtid() >> 5; q < n_sample; q += gstride() >> 5) {
        const int s = inv[sample[q]];
        int lo = 0, hi = ng - 1;  // the group holding sorted row s: last i_begin <= s
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (walks[mid].i_begin <= s) lo = mid;
            else hi = mid - 1;
        }
        const WalkDesc wd = walks[lo];
        const EpiDev ei = epi[s];
        double ax = 0, ay = 0, az = 0, pe = 0;
        int cnt = 0;
        for (int k = lane; k < wd.n_epj; k += 32) {
            const int id = id_epj[wd.epj_begin + k];
            const EpjMix e = epj[id];
            const double rsj = rs64[id];
            cnt += exact_neighbour(ei.x, ei.y, ei.z, ei.rs, e.x, e.y, e.z, rsj, eps2);
            const double dx = ei.x - e.x, dy = ei.y - e.y, dz = ei.z - e.z;
            const double r2e = dx * dx + dy * dy + dz * dz + eps2;
            const double r2c = r2e > wd.rcut2 ? r2e : wd.rcut2;
            const double ri = rsqrt(r2c);
            const double mr = m64[id] * ri;
            const double mr3 = mr * ri * ri;
            ax -= mr3 * dx;
            ay -= mr3 * dy;
            az -= mr3 * dz;
            pe -= mr;
        }
        for (int k = lane; k < wd.n_spj; k += 32) {
            const int id = id_spj[wd.spj_begin + k];
            const SpjMix j = spj[id];
            const SpjQ64 qq = spjq[id];
            const double rx = ei.x - j.x, ry = ei.y - j.y, rz = ei.z - j.z;
            const double r2 = rx * rx + ry * ry + rz * rz + eps2;
            const double qxx = qq.q[0], qyy = qq.q[1], qzz = qq.q[2], qxy = qq.q[3], qxz = qq.q[4], qyz = qq.q[5];
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
            const double A = qq.m * r3_inv - tr * r5_inv + 5.0 * qrr_r7;
            const double B = -2.0 * r5_inv;
            ax -= A * rx + B * qrx;
            ay -= A * ry + B * qry;
            az -= A * rz + B * qrz;
            pe -= qq.m * r_inv - 0.5 * tr * r3_inv + qrr_r5;
        }
        ax = warp_sum(ax);
        ay = warp_sum(ay);
        az = warp_sum(az);
        pe = warp_sum(pe);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        if (lane == 0) {
            SampleRec r;
            const Accp a = accp[s];
            r.acc[0] = a.x;
            r.acc[1] = a.y;
            r.acc[2] = a.z;
            r.pot = a.w;
            r.acc64[0] = G * ax;
            r.acc64[1] = G * ay;
            r.acc64[2] = G * az;
            r.pot64 = G * pe;
            r.n_ngb = nnb[s];
            r.n_ngb64 = cnt;
            r.step = slot;
            r.pad = 0;
            hist[(int64_t)slot * n_sample + q] = r;
        }
    }
}

__global__ void sample_advance_kernel(TreeHdr* h) {
    if (threadIdx.x == 0) h->sample_slot += 1;
}

// ---------------------------------------------------------------- host side

thread_local std::string t_error;

int nb_fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_error = buf;
    return code;
}

#define NB_CUDA(call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return nb_fail(PGF_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));      \
    } while (0)

template <class T>
struct DArr {
    T* d = nullptr;
    size_t n = 0;
    DArr() = default;
    DArr(const DArr&) = delete;
    DArr& operator=(const DArr&) = delete;
    ~DArr() { release(); }
    cudaError_t alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        cudaError_t e = cudaMalloc(&d, count * sizeof(T));
        if (e == cudaSuccess) n = count;
        else d = nullptr;
        return e;
    }
    void release() {
        if (d) cudaFree(d);
        d = nullptr;
        n = 0;
    }
};

}  // namespace
}  // namespace pgf

using namespace pgf;

static_assert(sizeof(pgf_nbody_sample) == sizeof(SampleRec), "pgf_nbody_sample layout");
static_assert(offsetof(pgf_nbody_sample, acc64) == offsetof(SampleRec, acc64), "pgf_nbody_sample layout");
static_assert(offsetof(pgf_nbody_sample, n_ngb) == offsetof(SampleRec, n_ngb), "pgf_nbody_sample layout");

struct pgf_nbody {
    int device = 0;
    int num_sms = 1;
    cudaStream_t stream = nullptr;
    int64_t n = 0;
    pgf_nbody_config cfg{};
    double inv_theta2 = 0.0;
    bool open_all = false;
    int variant = 0;
    // particle state, input order
    DArr<double> pos, vel, acc, pot, mass, rs;
    DArr<int32_t> n_ngb;
    // sort
    DArr<uint64_t> key_in, key_out;
    DArr<int32_t> val_in, order;
    // sorted copies
    DArr<EpiDev> epi;
    DArr<EpjMix> epj;
    DArr<double> epj_m64, epj_rs64;
    DArr<EpjF32> epj32;
    // cells
    int cap_cells = 0;
    DArr<TCell> cells;
    DArr<TCellW> cw;
    DArr<CMom> mom;
    DArr<int32_t> nch;
    DArr<int32_t> cell_order;  // cells by moments class (cell_bin)
    DArr<int4> bnd;  // per cell of the level being split: its octant ends (2 x 4)
    DArr<int32_t> blocksum;  // per-CTA child counts of one level, then their offsets
    DArr<SpjMix> spj;
    DArr<SpjF32> spj32;
    DArr<SpjQ64> spjq;
    // groups and walks
    DArr<int32_t> group_at, groups, cnt_e, cnt_s, bucket, queue;
    DArr<int32_t> inv_order;       // particle index -> sorted row
    DArr<int64_t> sample_idx;      // per-step sample: particles
    DArr<SampleRec> sample_hist;   // records [max_records][n_sample]
    int n_sample = 0, sample_records = 0;
    DArr<int32_t> front_at, fronts;  // frontier cells of the task split
    int front_limit = 1;              // frontier: topmost cells with at most this many particles
    int64_t cap_tasks = 0;
    DArr<int32_t> task_e, task_s;     // per (frontier, group) counts, then offsets
    DArr<WalkDesc> walks;
    int64_t cap_e = 0, cap_s = 0;
    DArr<int32_t> id_epj, id_spj;
    // force scratch and results
    DArr<Accp> out_accp;
    DArr<int32_t> out_nnb;
    DArr<int32_t> flags;  // [0] queue head, [1] n_retest, [2] kernel error word
    DArr<Retest> retest;
    int retest_cap = 1 << 20;
    DArr<TreeHdr> hdr;
    DArr<double> part;    // bbox partials
    DArr<double> energy;  // partials + result
    int bbox_blocks = 1;
    DArr<unsigned char> cub_tmp;
    size_t cub_bytes = 0;
    Params p{};
    // graph of the last captured run
    cudaGraphExec_t exec = nullptr;
    int graph_steps = 0;
    double graph_dt = 0.0;
    cudaEvent_t ev[6] = {};
    double last_tree_ms = 0, last_force_ms = 0;
    int64_t steps_done = 0;

    ~pgf_nbody() {
        if (exec) cudaGraphExecDestroy(exec);
        for (auto& e : ev)
            if (e) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace {

int grid_for(const pgf_nbody* h, int64_t work, int threads) {
    int64_t b = (work + threads - 1) / threads;
    const int64_t lim = (int64_t)h->num_sms * 8;
    if (b > lim) b = lim;
    if (b < 1) b = 1;
    return (int)b;
}

cudaError_t cub_sort(pgf_nbody* h, void* tmp, size_t& bytes) {
    return cub::DeviceRadixSort::SortPairs(tmp, bytes, h->key_in.d, h->key_out.d, h->val_in.d, h->order.d,
                                           (int64_t)h->n, 0, 3 * kMaxLevel, h->stream);
}

// Compacts the cell indices marked at their first particle (groups or
// frontier cells) into Morton order; the count goes to *count.
cudaError_t cub_select(pgf_nbody* h, void* tmp, size_t& bytes, const int32_t* at, int32_t* out, int32_t* count) {
    return cub::DeviceSelect::If(tmp, bytes, at, out, count, (int64_t)h->n, NonNegative(), h->stream);
}

// Tree, lists and work queue of the current positions (stream-ordered).
cudaError_t enqueue_build(pgf_nbody* h) {
    cudaStream_t s = h->stream;
    const int64_t n = h->n;
    TreeHdr* hd = h->hdr.d;
    bbox_partial_kernel<<<h->bbox_blocks, 256, 0, s>>>(h->pos.d, n, h->part.d);
    bbox_final_kernel<<<1, 256, 0, s>>>(h->part.d, h->bbox_blocks, n, hd, h->cells.d);
    cudaError_t e = cudaMemsetAsync(hd->hist, 0, sizeof(int32_t) * 2 * (kBuckets + kCellBins), s);
    if (e != cudaSuccess) return e;
    const int gn = grid_for(h, n, 256);
    keys_kernel<<<gn, 256, 0, s>>>(h->pos.d, n, hd, h->key_in.d, h->val_in.d);
    size_t bytes = h->cub_bytes;
    if ((e = cub_sort(h, h->cub_tmp.d, bytes)) != cudaSuccess) return e;
    gather_kernel<<<gn, 256, 0, s>>>(h->order.d, h->pos.d, h->mass.d, h->rs.d, n, h->epi.d, h->epj.d, h->epj_m64.d,
                                     h->epj_rs64.d, h->epj32.d, h->inv_order.d);
    const int gc = grid_for(h, h->cap_cells, 256);
    for (int L = 0; L < kLevels; ++L) {
        split_kernel<<<kLevelBlocks, 256, 0, s>>>(hd, h->cells.d, h->nch.d, h->bnd.d, h->blocksum.d, h->key_out.d, L,
                                                  h->cfg.n_leaf_limit);
        level_scan_kernel<<<1, kScanThreads, 0, s>>>(hd, h->blocksum.d, L, h->cap_cells);
        fill_kernel<<<kLevelBlocks, 256, 0, s>>>(hd, h->cells.d, h->nch.d, h->bnd.d, h->blocksum.d, L);
    }
    cell_hist_kernel<<<h->num_sms * 2, 256, 0, s>>>(hd, h->cells.d);
    cell_scan_kernel<<<1, 32, 0, s>>>(hd);
    cell_scatter_kernel<<<h->num_sms * 2, 256, 0, s>>>(hd, h->cells.d, h->cell_order.d);
    moments_kernel<true><<<gc, 256, 0, s>>>(hd, h->cells.d, h->cw.d, h->mom.d, h->epi.d, h->epj_m64.d, 0,
                                            h->inv_theta2, h->spj.d, h->spj32.d, h->spjq.d, h->cell_order.d);
    const int gm = h->num_sms * 2;
    for (int L = kLevels - 1; L >= 0; --L)
        moments_kernel<false><<<gm, 256, 0, s>>>(hd, h->cells.d, h->cw.d, h->mom.d, h->epi.d, h->epj_m64.d, L,
                                                 h->inv_theta2, h->spj.d, h->spj32.d, h->spjq.d, h->cell_order.d);
    if ((e = cudaMemsetAsync(h->group_at.d, 0xff, sizeof(int32_t) * n, s)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(h->front_at.d, 0xff, sizeof(int32_t) * n, s)) != cudaSuccess) return e;
    group_mark_kernel<<<gc, 256, 0, s>>>(hd, h->cells.d, h->group_at.d, h->cfg.n_group_limit);
    group_mark_kernel<<<gc, 256, 0, s>>>(hd, h->cells.d, h->front_at.d, h->front_limit);
    bytes = h->cub_bytes;
    if ((e = cub_select(h, h->cub_tmp.d, bytes, h->group_at.d, h->groups.d, &hd->n_groups)) != cudaSuccess) return e;
    bytes = h->cub_bytes;
    if ((e = cub_select(h, h->cub_tmp.d, bytes, h->front_at.d, h->fronts.d, &hd->n_fronts)) != cudaSuccess) return e;
    task_check_kernel<<<1, 32, 0, s>>>(hd, h->cap_tasks);
    const int gt = h->num_sms * 16;
    walk_task_count_kernel<<<gt, 128, 0, s>>>(hd, h->cw.d, h->cells.d, h->groups.d, h->fronts.d, h->task_e.d,
                                              h->task_s.d, h->open_all);
    group_reduce_kernel<<<grid_for(h, n, 128), 128, 0, s>>>(hd, h->cells.d, h->groups.d, h->walks.d, h->task_e.d,
                                                            h->task_s.d, h->cnt_e.d, h->cnt_s.d, h->bucket.d,
                                                            h->cfg.r_out * h->cfg.r_out);
    walk_scan_kernel<<<1, kScanThreads, 0, s>>>(hd, h->walks.d, h->cnt_e.d, h->cnt_s.d, h->cap_e, h->cap_s);
    walk_task_fill_kernel<<<gt, 128, 0, s>>>(hd, h->cw.d, h->cells.d, h->groups.d, h->fronts.d, h->walks.d,
                                             h->task_e.d, h->task_s.d, h->id_epj.d, h->id_spj.d, h->open_all);
    queue_scatter_kernel<<<grid_for(h, n, 256), 256, 0, s>>>(hd, h->bucket.d, h->queue.d);
    return cudaGetLastError();
}

cudaError_t enqueue_force(pgf_nbody* h) {
    if (h->cfg.precision == PGF_PRECISION_FP64) {
        cudaError_t e = launch_fp64(h->p, h->stream, h->num_sms);
        if (e == cudaSuccess) e = cudaMemsetAsync(h->p.n_retest, 0, sizeof(int32_t), h->stream);
        return e;
    }
    cudaError_t e = h->variant == 0 ? launch_mixed(h->p, h->stream, h->num_sms)
                                    : launch_ws(h->p, h->stream, h->num_sms, h->variant - 1, nullptr);
    if (e == cudaSuccess) e = launch_retest(h->p, h->stream, h->num_sms);
    return e;
}

cudaError_t enqueue_finish(pgf_nbody* h, double dt_kick) {
    if (h->n_sample > 0) {
        const int blocks = (int)std::min<int64_t>((h->n_sample + 3) / 4, (int64_t)h->num_sms * 8);
        sample_kernel<<<blocks, 128, 0, h->stream>>>(
            h->hdr.d, h->sample_idx.d, h->n_sample, h->inv_order.d, h->walks.d, h->epi.d, h->epj.d, h->epj_m64.d,
            h->epj_rs64.d, h->spj.d, h->spjq.d, h->id_epj.d, h->id_spj.d, h->cfg.eps2, h->cfg.G, h->out_accp.d,
            h->out_nnb.d, h->sample_hist.d, h->sample_records);
        sample_advance_kernel<<<1, 32, 0, h->stream>>>(h->hdr.d);
    }
    finish_kernel<<<grid_for(h, h->n, 256), 256, 0, h->stream>>>(h->hdr.d, h->order.d, h->out_accp.d, h->out_nnb.d,
                                                                 h->n, h->acc.d, h->pot.d, h->n_ngb.d, h->vel.d,
                                                                 dt_kick);
    return cudaGetLastError();
}

cudaError_t enqueue_step(pgf_nbody* h, double dt) {
    kick_drift_kernel<<<grid_for(h, 3 * h->n, 256), 256, 0, h->stream>>>(h->pos.d, h->vel.d, h->acc.d, 3 * h->n,
                                                                         0.5 * dt, dt);
    cudaError_t e = enqueue_build(h);
    if (e == cudaSuccess) e = enqueue_force(h);
    if (e == cudaSuccess) e = enqueue_finish(h, 0.5 * dt);
    return e;
}

int read_hdr(pgf_nbody* h, TreeHdr* out) {
    NB_CUDA(cudaMemcpy(out, h->hdr.d, sizeof(TreeHdr), cudaMemcpyDeviceToHost));
    return PGF_OK;
}

int check_errors(pgf_nbody* h) {
    TreeHdr t;
    if (int r = read_hdr(h, &t)) return r;
    int32_t kerr = 0;
    NB_CUDA(cudaMemcpy(&kerr, h->flags.d + 2, sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (t.err_sticky)
        return nb_fail(PGF_ERR_CAPACITY, "device list builder ran out of room (bits %d: 1 cells, 2 EPJ entries, "
                       "4 SPJ entries); raise list_capacity_factor", t.err_sticky);
    if (kerr) return nb_fail(PGF_ERR_DEVICE, "device error word %d", kerr);
    return PGF_OK;
}

void bind_params(pgf_nbody* h) {
    Params& p = h->p;
    p = Params{};
    p.epi = h->epi.d;
    p.epj = h->epj.d;
    p.epj_m64 = h->epj_m64.d;
    p.epj_rs64 = h->epj_rs64.d;
    p.spj = h->spj.d;
    p.spj_q64 = h->spjq.d;
    p.epj32 = h->epj32.d;
    p.spj32 = h->spj32.d;
    p.id_epj = h->id_epj.d;
    p.id_spj = h->id_spj.d;
    p.walks = h->walks.d;
    p.order = h->queue.d;
    p.n_walk = (int32_t)h->n;  // capacity; the build writes the count
    p.n_walk_dev = &h->hdr.d->n_walk;
    p.eps2 = h->cfg.eps2;
    p.G = h->cfg.G;
    p.out_accp = h->out_accp.d;
    p.out_nnb = h->out_nnb.d;
    p.queue_head = h->flags.d;
    p.n_retest = h->flags.d + 1;
    p.err = h->flags.d + 2;
    p.retest = h->retest.d;
    p.retest_cap = h->retest_cap;
}

cudaError_t alloc_cells(pgf_nbody* h, int cap) {
    h->cap_cells = cap;
    cudaError_t e;
    if ((e = h->cells.alloc(cap)) != cudaSuccess) return e;
    if ((e = h->cw.alloc(cap)) != cudaSuccess) return e;
    if ((e = h->mom.alloc(cap)) != cudaSuccess) return e;
    if ((e = h->nch.alloc(cap)) != cudaSuccess) return e;
    if ((e = h->cell_order.alloc(cap)) != cudaSuccess) return e;
    if ((e = h->bnd.alloc(2 * (size_t)cap)) != cudaSuccess) return e;
    if ((e = h->spj.alloc(cap)) != cudaSuccess) return e;
    if ((e = h->spj32.alloc(cap)) != cudaSuccess) return e;
    return h->spjq.alloc(cap);
}

cudaError_t alloc_tasks(pgf_nbody* h, int64_t cap) {
    h->cap_tasks = cap;
    cudaError_t e = h->task_e.alloc(cap);
    if (e == cudaSuccess) e = h->task_s.alloc(cap);
    return e;
}

void drop_graph(pgf_nbody* h) {
    if (h->exec) cudaGraphExecDestroy(h->exec);
    h->exec = nullptr;
    h->graph_steps = 0;
}

// Eager build at the current positions, growing the capacities until the
// tree and the lists fit (with the configured room on top).
int build_fit(pgf_nbody* h) {
    const double f = h->cfg.list_capacity_factor;
    for (int attempt = 0; attempt < 16; ++attempt) {
        NB_CUDA(cudaMemsetAsync(h->hdr.d, 0, sizeof(TreeHdr), h->stream));
        NB_CUDA(enqueue_build(h));
        NB_CUDA(cudaStreamSynchronize(h->stream));
        TreeHdr t;
        if (int r = read_hdr(h, &t)) return r;
        if (t.err == 0) {
            // Size every array to list_capacity_factor times what this build
            // used (growing or shrinking), then build again into the new
            // arrays; an array already within [1, 2] times that target stays.
            auto off = [](double cap, double target) { return cap < target || cap > 2.0 * target; };
            bool resized = false;
            const double tc = f * (double)t.level_begin[kLevels] + 64;
            if (off(h->cap_cells, tc)) {
                NB_CUDA(alloc_cells(h, (int)std::min<double>(std::ceil(tc), 1073741824.0)));
                resized = true;
            }
            const double te = f * (double)t.n_epj_entries + 1024;
            if (off((double)h->cap_e, te)) {
                h->cap_e = (int64_t)std::ceil(te);
                NB_CUDA(h->id_epj.alloc(h->cap_e));
                resized = true;
            }
            const double ts = f * (double)t.n_spj_entries + 1024;
            if (off((double)h->cap_s, ts)) {
                h->cap_s = (int64_t)std::ceil(ts);
                NB_CUDA(h->id_spj.alloc(h->cap_s));
                resized = true;
            }
            const double tt = f * (double)t.n_groups * (double)((t.n_fronts + kChunk - 1) / kChunk) + 1024;
            if (off((double)h->cap_tasks, tt)) {
                NB_CUDA(alloc_tasks(h, (int64_t)std::ceil(tt)));
                resized = true;
            }
            if (!resized) {
                NB_CUDA(cudaMemsetAsync(&h->hdr.d->err_sticky, 0, sizeof(int32_t), h->stream));
                return PGF_OK;
            }
            drop_graph(h);
            bind_params(h);
            continue;
        }
        if (t.err & kErrCells) {
            if (h->cap_cells >= 1 << 30) return nb_fail(PGF_ERR_CAPACITY, "more than 2^30 tree cells");
            NB_CUDA(alloc_cells(h, h->cap_cells * 2));
        }
        if (t.err & kErrEpj) {
            h->cap_e = (int64_t)(f * (double)t.n_epj_entries) + 1024;
            NB_CUDA(h->id_epj.alloc(h->cap_e));
        }
        if (t.err & kErrSpj) {
            h->cap_s = (int64_t)(f * (double)t.n_spj_entries) + 1024;
            NB_CUDA(h->id_spj.alloc(h->cap_s));
        }
        if (t.err & kErrTasks)
            NB_CUDA(alloc_tasks(h, (int64_t)(f * (double)t.n_groups * (double)((t.n_fronts + kChunk - 1) / kChunk)) + 1024));
        drop_graph(h);
        bind_params(h);
    }
    return nb_fail(PGF_ERR_CAPACITY, "device list builder did not fit after 16 attempts");
}

bool valid_variant(int v) {
    return v >= 0 && v < PGF_NUM_KERNEL_VARIANTS && !(v > 0 && ws_variant_uses_tma(v - 1));
}

}  // namespace

extern "C" {

const char* pgf_nbody_last_error(void) { return t_error.c_str(); }

int pgf_nbody_create(const pgf_nbody_config* cfg, int64_t n, const double* pos, const double* vel,
                     const double* mass, const double* r_search, pgf_nbody** out) {
    if (!cfg || !out || !pos || !vel || !mass || !r_search) return nb_fail(PGF_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (n <= 0) return nb_fail(PGF_ERR_ARG, "n must be positive");
    if (n > (int64_t)0x7fffffff) return nb_fail(PGF_ERR_CAPACITY, "more than 2^31-1 particles");
    if (cfg->n_leaf_limit < 1 || cfg->n_group_limit < 1) return nb_fail(PGF_ERR_ARG, "n_leaf_limit and n_group_limit must be >= 1");
    if (!(cfg->r_out > 0.0)) return nb_fail(PGF_ERR_ARG, "r_out must be positive");
    if (cfg->precision != PGF_PRECISION_MIXED && cfg->precision != PGF_PRECISION_FP64)
        return nb_fail(PGF_ERR_ARG, "unknown precision %d", cfg->precision);
    const int variant = cfg->kernel_variant < 0 ? PGF_DEFAULT_KERNEL_VARIANT : cfg->kernel_variant;
    if (!valid_variant(variant)) return nb_fail(PGF_ERR_ARG, "kernel variant %d is not available here", variant);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return nb_fail(PGF_ERR_NO_DEVICE, "no CUDA device");
    pgf_nbody* h = new (std::nothrow) pgf_nbody();
    if (!h) return nb_fail(PGF_ERR_CAPACITY, "out of host memory");
    auto bail = [&](int r) {
        pgf_nbody_destroy(h);
        return r;
    };
    h->cfg = *cfg;
    if (!(h->cfg.list_capacity_factor >= 1.0)) h->cfg.list_capacity_factor = 2.0;
    h->n = n;
    h->variant = variant;
    h->open_all = !(cfg->theta > 0.0);
    h->inv_theta2 = cfg->theta > 0 ? 1.0 / (cfg->theta * cfg->theta) : 0.0;
#define NB_TRY(call)                                                                           \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return bail(nb_fail(PGF_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_))); \
    } while (0)
    NB_TRY(cudaGetDevice(&h->device));
    NB_TRY(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device));
    NB_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    for (auto& e : h->ev) NB_TRY(cudaEventCreate(&e));
    const size_t n3 = 3 * (size_t)n;
    NB_TRY(h->pos.alloc(n3));
    NB_TRY(h->vel.alloc(n3));
    NB_TRY(h->acc.alloc(n3));
    NB_TRY(h->pot.alloc(n));
    NB_TRY(h->mass.alloc(n));
    NB_TRY(h->rs.alloc(n));
    NB_TRY(h->n_ngb.alloc(n));
    NB_TRY(h->key_in.alloc(n));
    NB_TRY(h->key_out.alloc(n));
    NB_TRY(h->val_in.alloc(n));
    NB_TRY(h->order.alloc(n));
    NB_TRY(h->epi.alloc(n));
    NB_TRY(h->epj.alloc(n));
    NB_TRY(h->epj_m64.alloc(n));
    NB_TRY(h->epj_rs64.alloc(n));
    NB_TRY(h->epj32.alloc(n));
    NB_TRY(alloc_cells(h, (int)std::min<int64_t>(4 * (n / (cfg->n_leaf_limit + 1)) + 1024, 1 << 30)));
    for (auto* a : {&h->group_at, &h->groups, &h->cnt_e, &h->cnt_s, &h->bucket, &h->queue, &h->front_at, &h->fronts,
                    &h->inv_order})
        NB_TRY(a->alloc(n));
    h->front_limit = (int)std::max<int64_t>(cfg->n_group_limit, n / 512);
    NB_TRY(alloc_tasks(h, 64 * (n / std::max(1, cfg->n_group_limit / 4) + 1) + 4096));
    NB_TRY(h->walks.alloc(n));
    h->cap_e = 8 * n + 1024;  // first guesses; the first build sizes them
    h->cap_s = 8 * n + 1024;
    NB_TRY(h->id_epj.alloc(h->cap_e));
    NB_TRY(h->id_spj.alloc(h->cap_s));
    NB_TRY(h->blocksum.alloc(kLevelBlocks));
    NB_TRY(h->out_accp.alloc(n));
    NB_TRY(h->out_nnb.alloc(n));
    NB_TRY(h->flags.alloc(8));
    NB_TRY(h->retest.alloc(h->retest_cap));
    NB_TRY(h->hdr.alloc(1));
    h->bbox_blocks = (int)std::min<int64_t>((n + 255) / 256, 1024);
    NB_TRY(h->part.alloc(6 * (size_t)h->bbox_blocks));
    NB_TRY(h->energy.alloc(2 * kEnergyBlocks + 2));
    {
        size_t b1 = 0, b2 = 0;
        NB_TRY(cub_sort(h, nullptr, b1));
        NB_TRY(cub_select(h, nullptr, b2, h->group_at.d, h->groups.d, &h->hdr.d->n_groups));
        h->cub_bytes = std::max(b1, b2);
        NB_TRY(h->cub_tmp.alloc(h->cub_bytes));
    }
    NB_TRY(cudaMemsetAsync(h->flags.d, 0, 8 * sizeof(int32_t), h->stream));
    NB_TRY(cudaMemsetAsync(h->acc.d, 0, n3 * sizeof(double), h->stream));
    NB_TRY(cudaMemcpyAsync(h->pos.d, pos, n3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    NB_TRY(cudaMemcpyAsync(h->vel.d, vel, n3 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    NB_TRY(cudaMemcpyAsync(h->mass.d, mass, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    NB_TRY(cudaMemcpyAsync(h->rs.d, r_search, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
#undef NB_TRY
    bind_params(h);
    if (int r = build_fit(h)) return bail(r);
    if (int r = pgf_nbody_force(h)) return bail(r);
    *out = h;
    return PGF_OK;
}

// Clears the sticky build error and the kernels' error word before a call.
static int clear_errors(pgf_nbody* h) {
    NB_CUDA(cudaMemsetAsync(&h->hdr.d->err_sticky, 0, sizeof(int32_t), h->stream));
    NB_CUDA(cudaMemsetAsync(h->flags.d + 2, 0, sizeof(int32_t), h->stream));
    return PGF_OK;
}

static int force_once(pgf_nbody* h) {
    if (int r = clear_errors(h)) return r;
    NB_CUDA(cudaEventRecord(h->ev[0], h->stream));
    NB_CUDA(enqueue_build(h));
    NB_CUDA(cudaEventRecord(h->ev[1], h->stream));
    NB_CUDA(enqueue_force(h));
    NB_CUDA(cudaEventRecord(h->ev[2], h->stream));
    NB_CUDA(enqueue_finish(h, 0.0));
    NB_CUDA(cudaStreamSynchronize(h->stream));
    float a = 0, b = 0;
    cudaEventElapsedTime(&a, h->ev[0], h->ev[1]);
    cudaEventElapsedTime(&b, h->ev[1], h->ev[2]);
    h->last_tree_ms = a;
    h->last_force_ms = b;
    return check_errors(h);
}

int pgf_nbody_force(pgf_nbody* h) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    int r = force_once(h);
    if (r != PGF_ERR_CAPACITY) return r;
    // The lists outgrew their arrays: grow them (dropping any captured
    // graph, which holds the old addresses) and evaluate again.
    if ((r = build_fit(h)) != PGF_OK) return r;
    return force_once(h);
}

int pgf_nbody_run(pgf_nbody* h, int n_steps, double dt, int use_graph, double* ms) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    if (n_steps < 0) return nb_fail(PGF_ERR_ARG, "negative step count");
    if (n_steps == 0) {
        if (ms) *ms = 0.0;
        return PGF_OK;
    }
    if (use_graph && (!h->exec || h->graph_steps != n_steps || h->graph_dt != dt)) {
        if (h->exec) {
            cudaGraphExecDestroy(h->exec);
            h->exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        NB_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < n_steps && e == cudaSuccess; ++k) e = enqueue_step(h, dt);
        cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return nb_fail(PGF_ERR_CUDA, "graph capture failed: %s",
                           cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        e = cudaGraphInstantiate(&h->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            h->exec = nullptr;
            return nb_fail(PGF_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
        }
        h->graph_steps = n_steps;
        h->graph_dt = dt;
    }
    if (int r = clear_errors(h)) return r;
    NB_CUDA(cudaEventRecord(h->ev[3], h->stream));
    if (use_graph) {
        NB_CUDA(cudaGraphLaunch(h->exec, h->stream));
    } else {
        for (int k = 0; k < n_steps; ++k) NB_CUDA(enqueue_step(h, dt));
    }
    NB_CUDA(cudaEventRecord(h->ev[4], h->stream));
    NB_CUDA(cudaStreamSynchronize(h->stream));
    float t = 0;
    cudaEventElapsedTime(&t, h->ev[3], h->ev[4]);
    if (ms) *ms = t;
    h->steps_done += n_steps;
    return check_errors(h);
}

int pgf_nbody_get(pgf_nbody* h, double* pos, double* vel, double* acc, double* pot, int32_t* n_ngb) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    const size_t n = (size_t)h->n;
    if (pos) NB_CUDA(cudaMemcpy(pos, h->pos.d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
    if (vel) NB_CUDA(cudaMemcpy(vel, h->vel.d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
    if (acc) NB_CUDA(cudaMemcpy(acc, h->acc.d, 3 * n * sizeof(double), cudaMemcpyDeviceToHost));
    if (pot) NB_CUDA(cudaMemcpy(pot, h->pot.d, n * sizeof(double), cudaMemcpyDeviceToHost));
    if (n_ngb) NB_CUDA(cudaMemcpy(n_ngb, h->n_ngb.d, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
    return PGF_OK;
}

int pgf_nbody_set_state(pgf_nbody* h, const double* pos, const double* vel) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    const size_t n = (size_t)h->n;
    if (pos) NB_CUDA(cudaMemcpy(h->pos.d, pos, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
    if (vel) NB_CUDA(cudaMemcpy(h->vel.d, vel, 3 * n * sizeof(double), cudaMemcpyHostToDevice));
    return PGF_OK;
}

int pgf_nbody_energy(pgf_nbody* h, double* kinetic, double* potential) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    const double self_coef = h->cfg.G / h->cfg.r_out;
    energy_partial_kernel<<<kEnergyBlocks, 256, 0, h->stream>>>(h->vel.d, h->mass.d, h->pot.d, h->n, self_coef,
                                                                 h->energy.d);
    energy_final_kernel<<<1, 32, 0, h->stream>>>(h->energy.d, kEnergyBlocks, h->energy.d + 2 * kEnergyBlocks);
    NB_CUDA(cudaGetLastError());
    double r[2];
    NB_CUDA(cudaMemcpyAsync(r, h->energy.d + 2 * kEnergyBlocks, sizeof(r), cudaMemcpyDeviceToHost, h->stream));
    NB_CUDA(cudaStreamSynchronize(h->stream));
    if (kinetic) *kinetic = r[0];
    if (potential) *potential = r[1];
    return PGF_OK;
}

int pgf_nbody_get_stats(pgf_nbody* h, pgf_nbody_stats* s) {
    if (!h || !s) return nb_fail(PGF_ERR_ARG, "NULL argument");
    TreeHdr t;
    if (int r = read_hdr(h, &t)) return r;
    s->n_cells = t.level_begin[kLevels];
    s->n_groups = t.n_groups;
    s->n_epj_entries = t.n_epj_entries;
    s->n_spj_entries = t.n_spj_entries;
    s->interactions_epep = (int64_t)t.n_epep;
    s->interactions_epsp = (int64_t)t.n_epsp;
    s->total_epep = (int64_t)t.total_epep;
    s->total_epsp = (int64_t)t.total_epsp;
    s->steps = h->steps_done;
    s->last_tree_ms = h->last_tree_ms;
    s->last_force_ms = h->last_force_ms;
    s->kernel_variant = h->variant;
    s->cap_cells = h->cap_cells;
    s->cap_epj_entries = h->cap_e;
    s->cap_spj_entries = h->cap_s;
    return PGF_OK;
}

int pgf_nbody_export_lists(pgf_nbody* h, int64_t* order, int64_t* group_begin, int64_t* epj_disp,
                           int64_t* spj_disp, int32_t* id_epj, int32_t* id_spj, double* cell_mass,
                           double* cell_pos, double* cell_quad, int32_t* cell_level) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    TreeHdr t;
    if (int r = read_hdr(h, &t)) return r;
    if (t.err) return nb_fail(PGF_ERR_STATE, "the last build failed (bits %d)", t.err);
    const int64_t n = h->n, ng = t.n_groups, nc = t.level_begin[kLevels];
    if (order) {
        std::vector<int32_t> o(n);
        NB_CUDA(cudaMemcpy(o.data(), h->order.d, n * sizeof(int32_t), cudaMemcpyDeviceToHost));
        for (int64_t i = 0; i < n; ++i) order[i] = o[i];
    }
    if (group_begin || epj_disp || spj_disp) {
        std::vector<WalkDesc> w(ng);
        if (ng) NB_CUDA(cudaMemcpy(w.data(), h->walks.d, ng * sizeof(WalkDesc), cudaMemcpyDeviceToHost));
        for (int64_t g = 0; g < ng; ++g) {
            if (group_begin) group_begin[g] = w[g].i_begin;
            if (epj_disp) epj_disp[g] = w[g].epj_begin;
            if (spj_disp) spj_disp[g] = w[g].spj_begin;
        }
        if (group_begin) group_begin[ng] = n;
        if (epj_disp) epj_disp[ng] = t.n_epj_entries;
        if (spj_disp) spj_disp[ng] = t.n_spj_entries;
    }
    if (id_epj && t.n_epj_entries)
        NB_CUDA(cudaMemcpy(id_epj, h->id_epj.d, t.n_epj_entries * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (id_spj && t.n_spj_entries)
        NB_CUDA(cudaMemcpy(id_spj, h->id_spj.d, t.n_spj_entries * sizeof(int32_t), cudaMemcpyDeviceToHost));
    if (cell_mass || cell_pos || cell_quad || cell_level) {
        std::vector<CMom> m(nc);
        std::vector<TCell> c(nc);
        NB_CUDA(cudaMemcpy(m.data(), h->mom.d, nc * sizeof(CMom), cudaMemcpyDeviceToHost));
        NB_CUDA(cudaMemcpy(c.data(), h->cells.d, nc * sizeof(TCell), cudaMemcpyDeviceToHost));
        for (int64_t k = 0; k < nc; ++k) {
            if (cell_mass) cell_mass[k] = m[k].m;
            for (int d = 0; d < 3; ++d)
                if (cell_pos) cell_pos[3 * k + d] = c[k].com[d];
            for (int q = 0; q < 6; ++q)
                if (cell_quad) cell_quad[6 * k + q] = m[k].q[q];
            if (cell_level) cell_level[k] = c[k].level;
        }
    }
    return PGF_OK;
}

int pgf_nbody_autotune(pgf_nbody* h, int repeats, int* best_variant, double* best_ms) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    if (h->cfg.precision != PGF_PRECISION_MIXED) return nb_fail(PGF_ERR_STATE, "autotune needs mixed precision");
    if (repeats < 1) repeats = 1;
    int best = h->variant;
    double best_t = 1e300;
    for (int v = 0; v < PGF_NUM_KERNEL_VARIANTS; ++v) {
        if (!valid_variant(v)) continue;
        h->variant = v;
        NB_CUDA(enqueue_force(h));  // warm-up
        NB_CUDA(cudaEventRecord(h->ev[0], h->stream));
        for (int r = 0; r < repeats; ++r) NB_CUDA(enqueue_force(h));
        NB_CUDA(cudaEventRecord(h->ev[1], h->stream));
        NB_CUDA(cudaStreamSynchronize(h->stream));
        float t = 0;
        cudaEventElapsedTime(&t, h->ev[0], h->ev[1]);
        if (t / repeats < best_t) {
            best_t = t / repeats;
            best = v;
        }
    }
    h->variant = best;
    if (h->exec) {
        cudaGraphExecDestroy(h->exec);
        h->exec = nullptr;
    }
    if (best_variant) *best_variant = best;
    if (best_ms) *best_ms = best_t;
    NB_CUDA(enqueue_force(h));
    NB_CUDA(enqueue_finish(h, 0.0));
    NB_CUDA(cudaStreamSynchronize(h->stream));
    return check_errors(h);
}

int pgf_nbody_set_group_limit(pgf_nbody* h, int n_group_limit) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    if (n_group_limit < 1) return nb_fail(PGF_ERR_ARG, "n_group_limit must be >= 1");
    NB_CUDA(cudaStreamSynchronize(h->stream));
    h->cfg.n_group_limit = n_group_limit;
    h->front_limit = (int)std::max<int64_t>(n_group_limit, h->n / 512);
    drop_graph(h);  // the captured steps build other lists now
    if (int r = build_fit(h)) return r;
    return pgf_nbody_force(h);
}

int pgf_nbody_autotune_groups(pgf_nbody* h, const int* limits, int n_limits, int repeats, double* step_ms,
                              int64_t* interactions, int* best_limit, int* best_variant, double* best_ms) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    if (n_limits < 0 || (n_limits > 0 && !limits)) return nb_fail(PGF_ERR_ARG, "bad candidate list");
    static const int kDefault[4] = {256, 512, 1024, 2048};
    if (n_limits == 0) {
        limits = kDefault;
        n_limits = 4;
    }
    if (repeats < 1) repeats = 1;
    int best = h->cfg.n_group_limit, best_v = h->variant;
    double best_t = 1e300;
    for (int c = 0; c < n_limits; ++c) {
        if (int r = pgf_nbody_set_group_limit(h, limits[c])) return r;
        if (h->cfg.precision == PGF_PRECISION_MIXED) {
            if (int r = pgf_nbody_autotune(h, repeats, nullptr, nullptr)) return r;
        }
        // Tree, lists and force of one evaluation at the current positions.
        NB_CUDA(enqueue_build(h));
        NB_CUDA(enqueue_force(h));
        NB_CUDA(cudaEventRecord(h->ev[0], h->stream));
        for (int r = 0; r < repeats; ++r) {
            NB_CUDA(enqueue_build(h));
            NB_CUDA(enqueue_force(h));
        }
        NB_CUDA(cudaEventRecord(h->ev[1], h->stream));
        NB_CUDA(cudaStreamSynchronize(h->stream));
        if (int r = check_errors(h)) return r;
        float t = 0;
        cudaEventElapsedTime(&t, h->ev[0], h->ev[1]);
        const double ms = t / repeats;
        TreeHdr th;
        if (int r = read_hdr(h, &th)) return r;
        if (step_ms) step_ms[c] = ms;
        if (interactions) interactions[c] = (int64_t)th.n_epep + (int64_t)th.n_epsp;
        if (ms < best_t) {
            best_t = ms;
            best = limits[c];
            best_v = h->variant;
        }
    }
    if (int r = pgf_nbody_set_group_limit(h, best)) return r;
    h->variant = best_v;
    if (best_limit) *best_limit = best;
    if (best_variant) *best_variant = best_v;
    if (best_ms) *best_ms = best_t;
    return pgf_nbody_force(h);
}

int pgf_nbody_set_sample(pgf_nbody* h, int n_sample, const int64_t* particles, int max_records) {
    if (!h) return nb_fail(PGF_ERR_ARG, "NULL handle");
    if (n_sample < 0 || max_records < 0 || (n_sample > 0 && (!particles || max_records == 0)))
        return nb_fail(PGF_ERR_ARG, "bad sample arguments");
    for (int q = 0; q < n_sample; ++q)
        if (particles[q] < 0 || particles[q] >= h->n) return nb_fail(PGF_ERR_ARG, "sample particle %d out of range", q);
    NB_CUDA(cudaStreamSynchronize(h->stream));
    drop_graph(h);  // the captured steps change
    h->n_sample = 0;
    h->sample_records = 0;
    if (n_sample == 0) return PGF_OK;
    NB_CUDA(h->sample_idx.alloc(n_sample));
    NB_CUDA(h->sample_hist.alloc((size_t)n_sample * max_records));
    NB_CUDA(cudaMemcpy(h->sample_idx.d, particles, n_sample * sizeof(int64_t), cudaMemcpyHostToDevice));
    NB_CUDA(cudaMemset(h->sample_hist.d, 0, (size_t)n_sample * max_records * sizeof(SampleRec)));
    NB_CUDA(cudaMemset(&h->hdr.d->sample_slot, 0, sizeof(int32_t)));
    h->n_sample = n_sample;
    h->sample_records = max_records;
    return PGF_OK;
}

int pgf_nbody_get_sample(pgf_nbody* h, int* n_records, pgf_nbody_sample* out) {
    if (!h || !n_records) return nb_fail(PGF_ERR_ARG, "NULL argument");
    NB_CUDA(cudaStreamSynchronize(h->stream));
    TreeHdr t;
    if (int r = read_hdr(h, &t)) return r;
    const int n = std::min(t.sample_slot, h->sample_records);
    *n_records = n;
    if (out && n > 0 && h->n_sample > 0)
        NB_CUDA(cudaMemcpy(out, h->sample_hist.d, (size_t)n * h->n_sample * sizeof(SampleRec), cudaMemcpyDeviceToHost));
    return PGF_OK;
}

int pgf_nbody_destroy(pgf_nbody* h) {
    if (!h) return PGF_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    delete h;
    return PGF_OK;
}

}  // extern "C"
