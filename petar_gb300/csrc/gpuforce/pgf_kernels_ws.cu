// Warp-specialised mixed-precision soft-force kernel for sm_103a.
//
// Same pair arithmetic, precision scheme and outputs as mixed_kernel
// (pgf_kernels_mixed.cu): walk-relative coordinates formed in FP64 and rounded
// to FP32, near EPJ with hi/lo coordinates, the linear cutoff and the exact
// neighbour count, far EPJ as plain gravity, EP-SP with the traceless
// quadrupole, FP32 partial sums flushed into FP64.  The difference is the
// data flow inside a CTA:
//
// * One producer warp walks the work queue.  For every walk pass it emits a
//   PASS_BEGIN item, then one item per j tile, then PASS_END.  For a tile it
//   gathers the EPJ/SPJ records through the id list (L2-resident), forms x - c
//   in FP64, classifies near/far, compacts with warp ballots and writes the
//   FP32 tile into a slot of a shared-memory ring.
// * CW consumer warps take the items in order.  They never stage data and
//   never wait for each other inside a pass: each waits only for the slot it
//   needs (mbarrier "full") and releases it when done (mbarrier "empty").  The
//   producer therefore runs ahead, across walk boundaries, by up to NS
//   items.
// * The producer works in FP32 only.  j positions arrive as (hi, lo) FP32
//   pairs (EpjF32 / SpjF32); x - c is (x_hi - c_hi) + (x_lo - c_lo), and for
//   near entries an error-free two-sum gives the walk-relative (hi, lo) pair.
//   GB300 runs FP64 at 1/64 of the FP32 rate, so FP64 conversion in the
//   producer would throttle it on small walks.
// * Consumers flush their FP32 partial sums into (hi, lo) FP32 accumulators
//   in shared memory with a two-sum (no FP64 in the pair loops either); the
//   j-slices are combined in FP64 once per pass.
// * Ambiguous neighbour pairs (within the guard band of r_search) are pushed
//   one by one as Retest records with their own list index, so no thread has
//   to coordinate its counts with another.
// * Every mbarrier wait is bounded by 1 s of %globaltimer; on expiry the thread
//   sets the device error word and returns.  The host reports PGF_ERR_DEVICE.
#include "pgf_internal.cuh"

#include <cuda.h>

namespace pgf {
namespace {

// Ring geometry is a template parameter of each variant: TE EPJ entries per
// EP tile (TE / 32 per producer lane), TE SPJ entries per SP tile (TE / 2
// with TMA staging), NS ring slots.
constexpr int kFlush = 256;   // pairs per consumer thread between FP64 flushes
constexpr int kKMax = 1 << 22;
constexpr unsigned long long kWaitLimitNs = 1000000000ull;
constexpr int kErrWaitTimeout = 1;

enum : int { kItemEP = 0, kItemSP = 1, kItemBegin = 2, kItemEnd = 3, kItemExit = 4 };

__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// Guard band in ulps of rs2 for the near-pair neighbour test of one i at
// distance D (max norm) from the walk centre; see kband_near in
// pgf_kernels_mixed.cu for the derivation: the FP32 test is off by less than
// 8 + 1.3e-6 D / r_ref ulps, r_ref = sqrt(rs^2 - eps2), and the band is
// 48 + 1e-5 D / r_ref.  Evaluated here in FP32 (GB300's FP64 pipe runs at
// 1/64 of the FP32 rate and this runs for every i of every pass); the few
// ulps of rounding of the FP32 form are far inside the factor of six between
// the band and the bound, and a larger band only adds FP64 re-tests.
__device__ __forceinline__ int kband_near(float D, float rs2, float eps2) {
    const float r2ref = rs2 - eps2;
    if (!(r2ref > 0.f)) return kKMax;
    const float k = 48.f + 1e-5f * D * rsqrt_approx(r2ref) * 1.001f;
    return k >= float(kKMax) ? kKMax : int(k) + 1;
}

// L2 policy for data read once per launch (the id lists): evicted before
// lines loaded with the default policy, so the streamed ids do not push the
// EPJ/SPJ records (re-read by every walk) out of L2.
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
    uint64_t pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ int ld_streamed(const int32_t* a, uint64_t pol) {
    int v;
    asm volatile("ld.global.nc.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}

// Error-free sum: s + e == a + b exactly (round-to-nearest, no reassociation).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(bar))
        : "memory");
}

// Waits for the phase of the given parity to complete; false after `limit_ns`
// of %globaltimer (1 s when 0), with the error word set.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int32_t* err, uint64_t limit_ns) {
    const unsigned long long limit = limit_ns ? limit_ns : kWaitLimitNs;
    const uint32_t a = smem_addr(bar);
    unsigned done = 0;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
    const unsigned long long t0 = globaltimer();
    for (;;) {
        // Suspend (up to the hint, 100 us) until the phase completes, so
        // that waiting warps leave the issue slots to the warps that work.
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(100000u)
            : "memory");
        if (done) return true;
        if (globaltimer() - t0 > limit) {
            atomicOr(err, kErrWaitTimeout);
            return false;
        }
    }
}

// mbarrier arrival that also expects `bytes` of asynchronous (TMA) writes.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_addr(bar)),
        "r"(bytes)
        : "memory");
}

// TMA gather of four rows (r0..r3) of a 2-D tensor map whose box is one row
// high, into consecutive rows at smem_dst; completion is signalled on bar.
// The rows must lie inside the tensor; the column coordinate is 0.
__device__ __forceinline__ void tma_gather4(void* smem_dst, const CUtensorMap* map, int r0, int r1, int r2, int r3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile::gather4.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(smem_addr(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(r0), "r"(r1), "r"(r2), "r"(r3), "r"(smem_addr(bar))
        : "memory");
}

// Named barrier among the consumer warps only (the producer never joins).
__device__ __forceinline__ void consumers_sync(int n_threads) {
    asm volatile("bar.sync 1, %0;" ::"r"(n_threads) : "memory");
}

// Scalar tiles: one float4 record per j.
template <int TE>
struct SlotEP {
    float4 nh[TE];  // near: hi x, y, z, m
    float4 nl[TE];  // near: lo x, y, z, rs2
    float4 fr[TE];  // far:  hi x, y, z, m
    int nidx[TE];   // near: entry index in the tile (for re-tests)
};
// SPJ tiles hold up to TE entries (TE / 2 with TMA staging): 48 bytes an
// entry, within the EP tile's 52, so they cost no shared memory.
template <int TE>
struct SlotSP {
    float4 sp[TE][3];
};
// Packed tiles: far EPJ and SPJ as pairs of j, component-interleaved, so a
// consumer reads (x0, x1), (y0, y1), ... as float2 operands of the FP32x2
// instructions.  An odd last entry is paired with a massless dummy at 1e15.
template <int TE>
struct SlotEPx2 {
    float4 nh[TE];
    float4 nl[TE];
    float4 fp[TE / 2][2];  // (x0 x1 y0 y1), (z0 z1 m0 m1)
    int nidx[TE];
};
template <int TE>
struct SlotSPx2 {
    float4 sp[TE / 2][6];  // x, y, z, m, -Qxx, -Qyy, -Qzz, -Qxy, -Qxz, -Qyz, -c (pairs), pad
};
template <bool PK, int TE>
union Slot {
    SlotEP<TE> ep;
    SlotSP<TE> sp;
};
template <int TE>
union Slot<true, TE> {
    SlotEPx2<TE> ep;
    SlotSPx2<TE> sp;
};
// Changeover mode: the EP slot also carries each near entry's changeover record.
template <int TE>
struct SlotEPco {
    float4 nh[TE];
    float4 nl[TE];
    float4 fr[TE];
    int nidx[TE];
    CoRec nco[TE];
};
template <int TE>
union SlotCo {
    SlotEPco<TE> ep;
    SlotSP<TE> sp;
};
template <int TE>
struct SlotEPx2co {
    float4 nh[TE];
    float4 nl[TE];
    float4 fp[TE / 2][2];
    int nidx[TE];
    CoRec nco[TE];
};
template <int TE>
union SlotCox2 {
    SlotEPx2co<TE> ep;
    SlotSPx2<TE> sp;
};
// What a kernel computes: soft force, neighbour search, or soft force with the
// changeover correction of neighbours fused in (scalar arithmetic only).
enum : int { kModeForce = 0, kModeSearch = 1, kModeChangeover = 2 };
template <bool PK, int TE, int MD>
struct SlotSel {
    using type = Slot<PK, TE>;
};
template <int TE>
struct SlotSel<false, TE, kModeChangeover> {
    using type = SlotCo<TE>;
};
template <int TE>
struct SlotSel<true, TE, kModeChangeover> {
    using type = SlotCox2<TE>;
};
template <int KI, int CT, bool CO>
struct CoExtra {};
// TMA staging of the producer: two 4 KB buffers (one 128-entry EPJ tile of
// 32-byte records or one 64-entry SPJ tile of 64-byte records each) and their
// transaction barriers.
template <bool TM>
struct TmExtra {};
template <>
struct TmExtra<true> {
    alignas(128) unsigned char stage[2][4096];
    uint64_t bar[2];
};
template <int KI, int CT>
struct CoExtra<KI, CT, true> {
    float2 dtot[KI][CT];   // (hi, lo) flushed neighbour-pair partials of pot_tot
    float2 dsoft[KI][CT];  // the same for pot_soft
    CoRec coi[KI][CT];     // changeover record of each i
};
constexpr float kDummyPos = 1e15f;
struct Hdr {
    int kind;
    int nn;     // near entries (EP), entries (SP)
    int nf;     // far entries (EP)
    int walk;   // walk index (kItemBegin)
    int ipass;  // first i of the pass (kItemBegin)
    int pad;
    int64_t base;  // first list entry of the tile
};

template <int CW, int KI, bool PK, int TE, int NS, int MD, bool TM = false>
struct Smem {
    TmExtra<TM> tm;
    typename SlotSel<PK, TE, MD>::type slot[NS];
    Hdr hdr[NS];
    uint64_t full[NS];
    uint64_t empty[NS];
    float2 acc[KI][4][CW * 32];  // (hi, lo) FP32 accumulators of the flushed partials
    int cnt[KI][CW * 32];        // neighbour counts
    float4 nlo[KI][CW * 32];     // near-pair data of each i: lo x, y, z and r_search^2
    int nkb[KI][CW * 32];        // guard band of each i (ulps)
    CoExtra<KI, CW * 32, MD == kModeChangeover> co;
};

// k_acc = 1 - W_acc and k_pot = 1 - W_pot of the changeover functions
// (src/changeover.hpp:294-334) in FP32.  W_acc is within an ulp of 1 for x
// near 0 (r near r_in), so 1 - W_acc is not formed by subtraction: with
// y = 1 - x, the identity (1-x)^4 (1 + 4x + 10x^2 + 20x^3)
// = 1 - x^4 (1 + 4y + 10y^2 + 20y^3) gives
// 1 - W_acc = x^4 (1 + 4y + 10y^2 + 20y^3 - 35 coff y^4), accurate to a few
// ulps of itself.  1 - W_pot is coff x^5 (5x^3 - 20x^2 + 28x - 14) inside the
// changeover, 0 below r_in and 1 - pot_off r beyond r_out.
__device__ __forceinline__ void co_k_f32(float r, float r_in, float norm, float coff, float pot_off, float& kacc,
                                         float& kpot) {
    const float x = (r - r_in) * norm;
    const float xa = fminf(fmaxf(x, 0.f), 1.f);
    const float y = 1.f - xa;
    const float xa2 = xa * xa;
    const float y2 = y * y;
    kacc = (xa2 * xa2) * (1.f + 4.f * y + 10.f * y2 + 20.f * (y2 * y) - 35.f * coff * (y2 * y2));
    if (x >= 1.f) {
        kpot = 1.f - pot_off * r;
    } else if (x > 0.f) {
        const float x2 = x * x;
        const float x3 = x2 * x;
        kpot = coff * (x2 * x3) * (5.f * x3 - 20.f * x2 + 28.f * x - 14.f);
    } else {
        kpot = 0.f;
    }
}

// ---------------------------------------------------------------- producer

// SR (neighbour search): EPJ tiles only, near entries only; far entries can
// hold no neighbour and SPJ lists are skipped.
template <int CW, int KI, bool PK, int MD, int TE, int NS, bool TM>
__device__ void producer(const Params& p, Smem<CW, KI, PK, TE, NS, MD, TM>& s, int lane, const CUtensorMap& tme,
                         const CUtensorMap& tms) {
    constexpr bool SR = MD == kModeSearch, CO = MD == kModeChangeover;
    static_assert(!TM || (MD == kModeForce && TE == 128), "TMA staging: force mode, 128-entry EP tiles");
    constexpr int kMaxPass = CW * 32 * KI;
    constexpr int kTileEP = TE, kTileSP = TM ? TE / 2 : TE, kSlots = NS;
    constexpr int QE = TE / 32, QS = kTileSP / 32;  // EPJ and SPJ entries per lane and tile
    constexpr int QB = QE < 4 ? QE : 4, QSB = QS < 2 ? QS : 2;  // ... converted at a time
    static_assert(QE % QB == 0 && QS % QSB == 0, "tiles of whole sub-batches");
    static_assert(QS >= 1 && TE % 64 == 0, "EP tiles of a multiple of 64 entries");
    const float eps2 = (float)p.eps2;
    const uint64_t stream_pol = l2_evict_first_policy();
    unsigned item = 0;
    unsigned tm_phase = 0;     // parity of the two TMA staging barriers
    unsigned tm_inflight = 0;  // staging buffers with a gather issued and not yet waited for
    // On a failed wait: let this warp's gathers still in flight land (each
    // wait bounded) before the CTA's shared memory goes away.
    auto bail = [&]() {
        if constexpr (TM) {
            for (int b = 0; b < 2; ++b)
                if (tm_inflight & (1u << b)) (void)mbar_wait(&s.tm.bar[b], (tm_phase >> b) & 1u, p.err, p.wait_limit_ns);
        }
    };
    auto acquire = [&](int& sl) -> bool {
        // Test hook (pgf_test_stall_producer): stop publishing after the
        // given number of items, so that the consumers' bounded waits expire.
        if (p.stall_after_items > 0 && item >= (unsigned)p.stall_after_items) return false;
        sl = item % kSlots;
        const unsigned parity = ((item / kSlots) & 1u) ^ 1u;
        return mbar_wait(&s.empty[sl], parity, p.err, p.wait_limit_ns);
    };
    auto publish = [&](int sl) {
        __syncwarp();
        mbar_arrive(&s.full[sl]);  // 32 arrivals complete the phase
        ++item;
    };
    const int n_walk = walk_count(p);
    for (;;) {
        int w_q = 0;
        if (lane == 0) w_q = atomicAdd(p.queue_head, 1);
        w_q = __shfl_sync(0xffffffffu, w_q, 0);
        if (w_q >= n_walk) {
            int sl;
            if (!acquire(sl)) return bail();
            if (lane == 0) s.hdr[sl].kind = kItemExit;
            publish(sl);
            return;
        }
        const int widx = p.order[w_q];
        const WalkDesc wd = p.walks[widx];
        // Walk centre as an FP32 (hi, lo) pair.
        const float chx = (float)wd.cx, chy = (float)wd.cy, chz = (float)wd.cz;
        const float clx = (float)(wd.cx - (double)chx), cly = (float)(wd.cy - (double)chy),
                    clz = (float)(wd.cz - (double)chz);
        const float rcut2 = (float)wd.rcut2;
        const float rsmax2 = wd.rs_max * wd.rs_max;
        const float hmax = fmaxf(wd.hx, fmaxf(wd.hy, wd.hz));
        const int n_ept = (wd.n_epj + kTileEP - 1) / kTileEP;
        const int n_spt = SR ? 0 : (wd.n_spj + kTileSP - 1) / kTileSP;
        const int n_tiles = n_ept + n_spt;
        // TMA staging: tile u (EP tiles, then SP tiles) is gathered into
        // stage[u & 1] while tile u - 1 is converted.  Lane l gathers entries
        // 4l .. 4l + 3 (rows past the tile's end read row 0 and are ignored), so
        // every tile moves exactly 4096 bytes.
        auto tm_issue = [&](int u) {
            if constexpr (TM) {
                const int b = u & 1;
                const bool ep = u < n_ept;
                // the buffer's previous contents were read through the generic proxy
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                const int t = ep ? u : u - n_ept;
                const int64_t base = ep ? wd.epj_begin + (int64_t)t * kTileEP : wd.spj_begin + (int64_t)t * kTileSP;
                const int nt = ep ? min(kTileEP, wd.n_epj - t * kTileEP) : min(kTileSP, wd.n_spj - t * kTileSP);
                const int32_t* ids = ep ? p.id_epj : p.id_spj;
                const int n_lanes = ep ? kTileEP / 4 : kTileSP / 4;
                int r[4] = {0, 0, 0, 0};
                if (lane < n_lanes) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int e = 4 * lane + j;
                        r[j] = e < nt ? ld_streamed(ids + base + e, stream_pol) : 0;
                    }
                }
                if (lane == 0) mbar_arrive_expect_tx(&s.tm.bar[b], 4096u);
                __syncwarp();
                if (lane < n_lanes)
                    tma_gather4(s.tm.stage[b] + lane * (ep ? 128 : 256), ep ? &tme : &tms, r[0], r[1], r[2], r[3],
                                &s.tm.bar[b]);
                tm_inflight |= 1u << b;
            }
        };
        auto tm_wait = [&](int u) -> bool {
            if constexpr (TM) {
                const int b = u & 1;
                const bool ok = mbar_wait(&s.tm.bar[b], (tm_phase >> b) & 1u, p.err, p.wait_limit_ns);
                if (ok) {
                    tm_phase ^= 1u << b;
                    tm_inflight &= ~(1u << b);
                }
                return ok;
            } else {
                return true;
            }
        };
        for (int ipass = 0; ipass < wd.n_i; ipass += kMaxPass) {
            int sl;
            if (!acquire(sl)) return bail();
            if (lane == 0) {
                s.hdr[sl].kind = kItemBegin;
                s.hdr[sl].walk = widx;
                s.hdr[sl].ipass = ipass;
            }
            publish(sl);
            if constexpr (TM) {
                if (n_tiles > 0) tm_issue(0);
            }
            // EPJ tiles: ids and records, converted QB entries per lane at a
            // time (the producer's registers stay those of a 128-entry tile).
            for (int t = 0; t < n_ept; ++t) {
                const int64_t base = wd.epj_begin + (int64_t)t * kTileEP;
                const int nt = min(kTileEP, wd.n_epj - t * kTileEP);
                if constexpr (TM) {
                    if (t + 1 < n_tiles) tm_issue(t + 1);
                    if (!tm_wait(t)) return bail();
                }
                int nn = 0, nf = 0;
#pragma unroll
                for (int qb = 0; qb < QE; qb += QB) {
                int id[QB];
                float4 r0[QB], r1[QB];
                if constexpr (TM) {
                    const float4* st = reinterpret_cast<const float4*>(s.tm.stage[t & 1]);
#pragma unroll
                    for (int qq = 0; qq < QB; ++qq) {
                        const int e = (qb + qq) * 32 + lane;
                        id[qq] = e < nt ? 0 : -1;
                        r0[qq] = st[2 * e];
                        r1[qq] = st[2 * e + 1];
                    }
                } else {
#pragma unroll
                    for (int qq = 0; qq < QB; ++qq) {
                        const int e = (qb + qq) * 32 + lane;
                        id[qq] = e < nt ? ld_streamed(p.id_epj + base + e, stream_pol) : -1;
                    }
#pragma unroll
                    for (int qq = 0; qq < QB; ++qq) {
                        if (id[qq] >= 0) {
                            const float4* src = reinterpret_cast<const float4*>(p.epj32 + id[qq]);
                            r0[qq] = __ldg(src);
                            r1[qq] = __ldg(src + 1);
                        } else {
                            r0[qq] = r1[qq] = make_float4(0.f, 0.f, 0.f, 0.f);
                        }
                    }
                }
                if (qb == 0 && !acquire(sl)) return bail();
                auto& S = s.slot[sl].ep;
#pragma unroll
                for (int qq = 0; qq < QB; ++qq) {
                    const int q = qb + qq;
                    const int e = q * 32 + lane;
                    const bool valid = e < nt;
                    bool near = false;
                    float hx = 0.f, hy = 0.f, hz = 0.f, m = 0.f, rs2 = 0.f, lx = 0.f, ly = 0.f, lz = 0.f;
                    if (valid) {
                        // x - c to within about 1 ulp; exact (hi, lo) below for near entries
                        const float sx = r0[qq].x - chx, sy = r0[qq].y - chy, sz = r0[qq].z - chz;
                        const float tx = r1[qq].x - clx, ty = r1[qq].y - cly, tz = r1[qq].z - clz;
                        hx = sx + tx;
                        hy = sy + ty;
                        hz = sz + tz;
                        m = r0[qq].w;
                        rs2 = r1[qq].w;
                        const float ex = fmaxf(fabsf(hx) - wd.hx, 0.f);
                        const float ey = fmaxf(fabsf(hy) - wd.hy, 0.f);
                        const float ez = fmaxf(fabsf(hz) - wd.hz, 0.f);
                        const float dist2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
                        const float R = sqrtf(fmaxf(fmaxf(rsmax2, rs2), rcut2));
                        const float dmax = fmaxf(fabsf(hx), fmaxf(fabsf(hy), fabsf(hz)));
                        const float Rm = R * 1.001f + 1e-6f * (dmax + hmax);
                        near = !(dist2 > Rm * Rm);
                        if (near) {
                            // (x_hi - c_hi) exactly as s + e, then (s, e + x_lo - c_lo)
                            // renormalised: hi + lo = x - c to about 2^-48 |x|.
                            float s_, e_;
                            two_sum(r0[qq].x, -chx, s_, e_);
                            two_sum(s_, e_ + tx, hx, lx);
                            two_sum(r0[qq].y, -chy, s_, e_);
                            two_sum(s_, e_ + ty, hy, ly);
                            two_sum(r0[qq].z, -chz, s_, e_);
                            two_sum(s_, e_ + tz, hz, lz);
                        }
                    }
                    const unsigned bn = __ballot_sync(0xffffffffu, valid && near);
                    const unsigned bf = __ballot_sync(0xffffffffu, valid && !near && !SR);
                    const unsigned lt = (1u << lane) - 1u;
                    if (valid && near) {
                        const int pos = nn + __popc(bn & lt);
                        S.nh[pos] = make_float4(hx, hy, hz, m);
                        S.nl[pos] = make_float4(lx, ly, lz, rs2);
                        S.nidx[pos] = e;
                        if constexpr (CO) S.nco[pos] = p.epj_co[id[qq]];
                    } else if (valid && !SR) {
                        const int pos = nf + __popc(bf & lt);
                        if constexpr (PK) {
                            float* f = reinterpret_cast<float*>(&S.fp[pos >> 1][0]) + (pos & 1);
                            f[0] = hx;
                            f[2] = hy;
                            f[4] = hz;
                            f[6] = m;
                        } else {
                            S.fr[pos] = make_float4(hx, hy, hz, m);
                        }
                    }
                    nn += __popc(bn);
                    nf += __popc(bf);
                }
                }  // sub-batches
                auto& S = s.slot[sl].ep;
                if constexpr (PK && !SR) {
                    if ((nf & 1) && lane == 0) {
                        float* f = reinterpret_cast<float*>(&S.fp[nf >> 1][0]) + 1;
                        f[0] = f[2] = f[4] = kDummyPos;
                        f[6] = 0.f;
                    }
                }
                if (lane == 0) {
                    s.hdr[sl].kind = kItemEP;
                    s.hdr[sl].nn = nn;
                    s.hdr[sl].nf = nf;
                    s.hdr[sl].base = base;
                }
                publish(sl);
            }
            // SPJ tiles: 64-byte records, QSB entries per lane at a time.
            for (int t = 0; t < n_spt; ++t) {
                const int64_t base = wd.spj_begin + (int64_t)t * kTileSP;
                const int nt = min(kTileSP, wd.n_spj - t * kTileSP);
                if constexpr (TM) {
                    const int u = n_ept + t;
                    if (u + 1 < n_tiles) tm_issue(u + 1);
                    if (!tm_wait(u)) return bail();
                }
#pragma unroll
                for (int qb = 0; qb < QS; qb += QSB) {
                int id[QSB];
                float4 r[QSB][4];
                if constexpr (TM) {
                    const float4* st = reinterpret_cast<const float4*>(s.tm.stage[(n_ept + t) & 1]);
#pragma unroll
                    for (int qq = 0; qq < QSB; ++qq) {
                        const int e = (qb + qq) * 32 + lane;
#pragma unroll
                        for (int v = 0; v < 4; ++v) r[qq][v] = st[4 * e + v];
                    }
                } else {
#pragma unroll
                    for (int qq = 0; qq < QSB; ++qq) {
                        const int e = (qb + qq) * 32 + lane;
                        id[qq] = e < nt ? ld_streamed(p.id_spj + base + e, stream_pol) : -1;
                    }
#pragma unroll
                    for (int qq = 0; qq < QSB; ++qq) {
                        if (id[qq] >= 0) {
                            const float4* src = reinterpret_cast<const float4*>(p.spj32 + id[qq]);
#pragma unroll
                            for (int u = 0; u < 4; ++u) r[qq][u] = __ldg(src + u);
                        }
                    }
                }
                if (qb == 0 && !acquire(sl)) return bail();
                auto& S = s.slot[sl].sp;
#pragma unroll
                for (int qq = 0; qq < QSB; ++qq) {
                    const int q = qb + qq;
                    const int e = q * 32 + lane;
                    if (e < nt) {
                        // SpjF32: (xh yh zh m) (xl yl zl tr) (Qxx Qyy Qzz Qxy) (Qxz Qyz pad pad)
                        const float hx = (r[qq][0].x - chx) + (r[qq][1].x - clx);
                        const float hy = (r[qq][0].y - chy) + (r[qq][1].y - cly);
                        const float hz = (r[qq][0].z - chz) + (r[qq][1].z - clz);
                        const float m = r[qq][0].w;
                        const float c = -r[qq][1].w * eps2;
                        if constexpr (PK) {
                            float* f = reinterpret_cast<float*>(&S.sp[e >> 1][0]) + (e & 1);
                            f[0] = hx;
                            f[2] = hy;
                            f[4] = hz;
                            f[6] = m;
                            f[8] = -r[qq][2].x;
                            f[10] = -r[qq][2].y;
                            f[12] = -r[qq][2].z;
                            f[14] = -r[qq][2].w;
                            f[16] = -r[qq][3].x;
                            f[18] = -r[qq][3].y;
                            f[20] = -c;
                        } else {
                            S.sp[e][0] = make_float4(hx, hy, hz, m);
                            S.sp[e][1] = r[qq][2];
                            S.sp[e][2] = make_float4(r[qq][3].x, r[qq][3].y, c, 0.f);
                        }
                    }
                }
                }  // sub-batches
                auto& S = s.slot[sl].sp;
                if constexpr (PK) {
                    if ((nt & 1) && lane == 0) {
                        float* f = reinterpret_cast<float*>(&S.sp[nt >> 1][0]) + 1;
                        f[0] = f[2] = f[4] = kDummyPos;
                        for (int u = 6; u <= 20; u += 2) f[u] = 0.f;
                    }
                }
                if (lane == 0) {
                    s.hdr[sl].kind = kItemSP;
                    s.hdr[sl].nn = nt;
                    s.hdr[sl].nf = 0;
                    s.hdr[sl].base = base;
                }
                publish(sl);
            }
            if (!acquire(sl)) return bail();
            if (lane == 0) s.hdr[sl].kind = kItemEnd;
            publish(sl);
        }
    }
}

// ---------------------------------------------------------------- consumer

template <int N>
struct IntC {
    static constexpr int value = N;
};

// Issue cost per j entry of a pass of nip i-particles with ku i per thread on
// ct_threads consumer threads: warps that issue, times the pairs each thread
// runs per j, plus a small charge for the shared-memory load each j costs a
// thread, divided by the j-slices the pass splits a tile into.
__device__ __forceinline__ float pass_cost(int nip, int ku, int ct_threads) {
    const int S = (nip + ku - 1) / ku;
    const int n_js = ct_threads / S;
    if (n_js == 0) return 3.0e38f;
    const int warps = (n_js * S + 31) >> 5;
    return (float)warps * ((float)ku + 0.15f) / (float)n_js;
}

// Consumer registers hold only what the far and SP loops need: the i hi
// coordinates and the pair accumulators.  The near-only data of each i (lo
// coordinates, r_search^2, guard band) and the neighbour counts live in
// shared memory and are read once per tile that has near entries.
template <int CW, int KI, bool PK, int MD, int TE, int NS, bool TM>
__device__ void consumer(const Params& p, Smem<CW, KI, PK, TE, NS, MD, TM>& s, int ct) {
    constexpr bool SR = MD == kModeSearch, CO = MD == kModeChangeover;
    constexpr int kSlots = NS;
    constexpr int CT = CW * 32;
    constexpr int kMaxPass = CT * KI;
    constexpr int KA = KI > 1 ? KI - 1 : 1;  // the other i-per-thread count a pass may use
    const float eps2 = (float)p.eps2;
    unsigned item = 0;

    // Pass state.  A pass runs ku (KA or KI) i-particles per thread, whichever
    // leaves fewer lanes idle; the tile bodies are instantiated for both.
    float rcut2 = 0.f;
    int nip = 0, S = 1, n_js = 1, js = 0, slot = 0, ku = KI, gbase = 0;
    bool active = false;
    // Scalar path: i coordinates and accumulators a[0..2] acceleration, a[3]
    // potential.  Packed path: (-x_i, -x_i) operands and pair accumulators
    // b[0..2] acceleration, b[3] minus the potential.
    float xih[PK ? 1 : KI], yih[PK ? 1 : KI], zih[PK ? 1 : KI];
    float a[PK ? 1 : KI][4];
    float2 nx2[PK ? KI : 1], ny2[PK ? KI : 1], nz2[PK ? KI : 1];
    float2 b[PK ? KI : 1][4];
    // Changeover: pot_tot and pot_soft partials of neighbour pairs (all other
    // pairs add the same term to both, in a[k][3]).
    float dt[CO ? KI : 1], ds[CO ? KI : 1];
    double r_out_walk = 0.0, rcut2d = 0.0, self_scale = 1.0;
    int walk_cur = 0;
    int since = 0;
#pragma unroll
    for (int k = 0; k < (CO ? KI : 1); ++k) dt[k] = ds[k] = 0.f;
#pragma unroll
    for (int k = 0; k < (PK ? 1 : KI); ++k) {
        xih[k] = yih[k] = zih[k] = 0.f;
        a[k][0] = a[k][1] = a[k][2] = a[k][3] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < (PK ? KI : 1); ++k) {
        nx2[k] = ny2[k] = nz2[k] = make_float2(0.f, 0.f);
        b[k][0] = b[k][1] = b[k][2] = b[k][3] = make_float2(0.f, 0.f);
    }
    auto xi = [&](int k) -> float {
        if constexpr (PK) return -nx2[k].x; else return xih[k];
    };
    auto yi = [&](int k) -> float {
        if constexpr (PK) return -ny2[k].x; else return yih[k];
    };
    auto zi = [&](int k) -> float {
        if constexpr (PK) return -nz2[k].x; else return zih[k];
    };
    // Scalar accumulation used by the near loop in both paths.
    auto acc4 = [&](int k, float mri3, float dx, float dy, float dz, float mri) {
        if constexpr (PK) {
            b[k][0].x = fmaf(mri3, dx, b[k][0].x);
            b[k][1].x = fmaf(mri3, dy, b[k][1].x);
            b[k][2].x = fmaf(mri3, dz, b[k][2].x);
            b[k][3].x += mri;
        } else {
            a[k][0] = fmaf(mri3, dx, a[k][0]);
            a[k][1] = fmaf(mri3, dy, a[k][1]);
            a[k][2] = fmaf(mri3, dz, a[k][2]);
            a[k][3] -= mri;
        }
    };
    // Acceleration-only accumulation (changeover neighbour pairs).
    auto acc3 = [&](int k, float f, float dx, float dy, float dz) {
        if constexpr (PK) {
            b[k][0].x = fmaf(f, dx, b[k][0].x);
            b[k][1].x = fmaf(f, dy, b[k][1].x);
            b[k][2].x = fmaf(f, dz, b[k][2].x);
        } else {
            a[k][0] = fmaf(f, dx, a[k][0]);
            a[k][1] = fmaf(f, dy, a[k][1]);
            a[k][2] = fmaf(f, dz, a[k][2]);
        }
    };
    auto clear_acc = [&]() {
#pragma unroll
        for (int k = 0; k < KI; ++k) {
            if constexpr (PK) {
#pragma unroll
                for (int q = 0; q < 4; ++q) b[k][q] = make_float2(0.f, 0.f);
            } else {
#pragma unroll
                for (int q = 0; q < 4; ++q) a[k][q] = 0.f;
            }
            if constexpr (CO) dt[k] = ds[k] = 0.f;
        }
    };

    auto flush = [&]() {
#pragma unroll
        for (int k = 0; k < KI; ++k) {
            if (k >= ku) continue;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                float x;
                if constexpr (PK) {
                    x = b[k][q].x + b[k][q].y;
                    if (q == 3) x = -x;
                } else {
                    x = a[k][q];
                }
                float2 v = s.acc[k][q][ct];
                float e;
                two_sum(v.x, x, v.x, e);
                v.y += e;
                s.acc[k][q][ct] = v;
            }
            if constexpr (CO) {
                float2 v = s.co.dtot[k][ct];
                float e;
                two_sum(v.x, dt[k], v.x, e);
                v.y += e;
                s.co.dtot[k][ct] = v;
                v = s.co.dsoft[k][ct];
                two_sum(v.x, ds[k], v.x, e);
                v.y += e;
                s.co.dsoft[k][ct] = v;
            }
        }
        clear_acc();
        since = 0;
    };
    auto push_retest = [&](int k, int64_t jidx) -> int {
        const int gi = gbase + k * S;
        const int r = atomicAdd(p.n_retest, 1);
        if (r < p.retest_cap) {
            Retest rr;
            rr.j_begin = jidx;
            rr.i = gi;
            rr.n = 1;
            rr.walk = CO ? walk_cur : 0;  // only the changeover re-test reads it
            rr.pad = 0;
            p.retest[r] = rr;
            return 0;
        }
        const EpiDev ei = p.epi[gi];
        const int id = p.id_epj[jidx];
        const EpjMix e = p.epj[id];
        const int nb = exact_neighbour(ei.x, ei.y, ei.z, ei.rs, e.x, e.y, e.z, p.epj_rs64[id], p.eps2);
        if constexpr (CO) {
            // Capacity overflow: apply the changeover difference here.
            const CoRec ci = p.epi_co[gi], cj = p.epj_co[id];
            if (nb && ci.id != cj.id) {
                double d[5];
                co_pair_diff(ei, ci, e, e.m, cj, p.eps2, rcut2d, d);
                acc3(k, 1.f, (float)d[0], (float)d[1], (float)d[2]);
                dt[k] += (float)d[3];
                ds[k] += (float)d[4];
            }
        }
        return nb;
    };

    // One EPJ tile with KU i-particles per thread.
    auto ep_tile = [&](auto ku_c, const Hdr& h, int sl) {
        constexpr int KU = decltype(ku_c)::value;
        const auto& T = s.slot[sl].ep;
        const int pn = (h.nn + n_js - 1) / n_js;
        const int j0 = min(h.nn, js * pn);
        const int j1 = min(h.nn, j0 + pn);
        if (j1 > j0) {
            float4 lo[KU];
            int kb[KU], c[KU];
            bool vk[KU];
            CoRec ci[CO ? KU : 1];
#pragma unroll
            for (int k = 0; k < KU; ++k) {
                lo[k] = s.nlo[k][ct];
                kb[k] = s.nkb[k][ct];
                c[k] = 0;
                vk[k] = slot + k * S < nip;
                if constexpr (CO) ci[k] = s.co.coi[k][ct];
            }
            (void)ci;
#pragma unroll 1
            for (int j = j0; j < j1; ++j) {
                const float4 hh = T.nh[j];
                const float4 ll = T.nl[j];
#pragma unroll
                for (int k = 0; k < KU; ++k) {
                    const float dx = (hh.x - xi(k)) + (ll.x - lo[k].x);
                    const float dy = (hh.y - yi(k)) + (ll.y - lo[k].y);
                    const float dz = (hh.z - zi(k)) + (ll.z - lo[k].z);
                    float r2 = fmaf(dx, dx, eps2);
                    r2 = fmaf(dy, dy, r2);
                    r2 = fmaf(dz, dz, r2);
                    const float rs2 = fmaxf(lo[k].w, ll.w);
                    const int e = __float_as_int(r2) - __float_as_int(rs2) + kb[k];
                    c[k] += (int)((unsigned)e >> 31);
                    if ((unsigned)e < (unsigned)(2 * kb[k]) && vk[k]) c[k] += push_retest(k, h.base + T.nidx[j]);
                    if constexpr (CO) {
                        const CoRec& cj = T.nco[j];
                        if ((e < 0) && cj.id != ci[k].id) {
                            // neighbour: changeover force and potentials (src/hard.hpp:1404-1480
                            // composed with the linear-cutoff kernel term it replaces)
                            const float ri = rsqrt_approx(r2);
                            const float r = r2 * ri;
                            const bool use_i = ci[k].r_out > cj.r_out;
                            float kacc, kpot;
                            co_k_f32(r, use_i ? ci[k].r_in : cj.r_in, use_i ? ci[k].norm : cj.norm,
                                     use_i ? ci[k].coff : cj.coff, use_i ? ci[k].pot_off : cj.pot_off, kacc, kpot);
                            const float f = hh.w * kacc * (ri * ri * ri);
                            acc3(k, f, dx, dy, dz);
                            const float meri = cj.mass * ri;
                            dt[k] -= meri;
                            ds[k] = fmaf(-meri, kpot, ds[k]);
                        } else {
                            const float ri = rsqrt_approx(fmaxf(r2, rcut2));
                            const float mri = hh.w * ri;
                            acc4(k, mri * (ri * ri), dx, dy, dz, mri);
                        }
                    } else if constexpr (!SR) {
                        const float ri = rsqrt_approx(fmaxf(r2, rcut2));
                        const float mri = hh.w * ri;
                        acc4(k, mri * (ri * ri), dx, dy, dz, mri);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < KU; ++k) s.cnt[k][ct] += c[k];
        }
        int nfar = 0;
        if constexpr (SR) {
            // no far entries in a neighbour search
        } else if constexpr (PK) {
            // far pairs of j, two per FP32x2 instruction
            const int np = (h.nf + 1) >> 1;
            const int pp = (np + n_js - 1) / n_js;
            const int f0 = min(np, js * pp);
            const int f1 = min(np, f0 + pp);
            const float2 e2 = make_float2(eps2, eps2);
#pragma unroll 2
            for (int j = f0; j < f1; ++j) {
                const float4 u = T.fp[j][0];
                const float4 v = T.fp[j][1];
                const float2 X = make_float2(u.x, u.y), Y = make_float2(u.z, u.w);
                const float2 Z = make_float2(v.x, v.y), M = make_float2(v.z, v.w);
#pragma unroll
                for (int k = 0; k < KU; ++k) {
                    const float2 dx = __fadd2_rn(X, nx2[k]);
                    const float2 dy = __fadd2_rn(Y, ny2[k]);
                    const float2 dz = __fadd2_rn(Z, nz2[k]);
                    float2 r2 = __ffma2_rn(dx, dx, e2);
                    r2 = __ffma2_rn(dy, dy, r2);
                    r2 = __ffma2_rn(dz, dz, r2);
                    const float2 ri = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
                    const float2 mri = __fmul2_rn(M, ri);
                    const float2 mri3 = __fmul2_rn(mri, __fmul2_rn(ri, ri));
                    b[k][0] = __ffma2_rn(mri3, dx, b[k][0]);
                    b[k][1] = __ffma2_rn(mri3, dy, b[k][1]);
                    b[k][2] = __ffma2_rn(mri3, dz, b[k][2]);
                    b[k][3] = __fadd2_rn(b[k][3], mri);
                }
            }
            nfar = 2 * (f1 - f0);
        } else {
            const int pf = (h.nf + n_js - 1) / n_js;
            const int f0 = min(h.nf, js * pf);
            const int f1 = min(h.nf, f0 + pf);
#pragma unroll 4
            for (int j = f0; j < f1; ++j) {
                const float4 hh = T.fr[j];
#pragma unroll
                for (int k = 0; k < KU; ++k) {
                    const float dx = hh.x - xih[k];
                    const float dy = hh.y - yih[k];
                    const float dz = hh.z - zih[k];
                    float r2 = fmaf(dx, dx, eps2);
                    r2 = fmaf(dy, dy, r2);
                    r2 = fmaf(dz, dz, r2);
                    const float ri = rsqrt_approx(r2);
                    const float mri = hh.w * ri;
                    const float mri3 = mri * (ri * ri);
                    a[k][0] = fmaf(mri3, dx, a[k][0]);
                    a[k][1] = fmaf(mri3, dy, a[k][1]);
                    a[k][2] = fmaf(mri3, dz, a[k][2]);
                    a[k][3] -= mri;
                }
            }
            nfar = f1 - f0;
        }
        since += (j1 - j0) + nfar;
    };

    // One SPJ tile with KU i-particles per thread.
    auto sp_tile = [&](auto ku_c, const Hdr& h, int sl) {
        constexpr int KU = decltype(ku_c)::value;
        const auto& T = s.slot[sl].sp;
        if constexpr (PK) {
            const int np = (h.nn + 1) >> 1;
            const int pp = (np + n_js - 1) / n_js;
            const int j0 = min(np, js * pp);
            const int j1 = min(np, j0 + pp);
            const float2 e2 = make_float2(eps2, eps2);
#pragma unroll 1
            for (int j = j0; j < j1; ++j) {
                const float4 w0 = T.sp[j][0], w1 = T.sp[j][1], w2 = T.sp[j][2];
                const float4 w3 = T.sp[j][3], w4 = T.sp[j][4], w5 = T.sp[j][5];
                const float2 X = make_float2(w0.x, w0.y), Y = make_float2(w0.z, w0.w);
                const float2 Z = make_float2(w1.x, w1.y), M = make_float2(w1.z, w1.w);
                // nQ = -Q and nC = -c, so that the terms below need no negation:
                // with u = d.(-Q).d - c = -(d.Q.d + c) and t = u / r^5,
                // acc += (m/r^3 - 2.5 t/r^2) d + (-Q).d / r^5 and
                // -pot += m/r - 0.5 t.
                const float2 Qxx = make_float2(w2.x, w2.y), Qyy = make_float2(w2.z, w2.w);
                const float2 Qzz = make_float2(w3.x, w3.y), Qxy = make_float2(w3.z, w3.w);
                const float2 Qxz = make_float2(w4.x, w4.y), Qyz = make_float2(w4.z, w4.w);
                const float2 C = make_float2(w5.x, w5.y);
                const float2 km25 = make_float2(-2.5f, -2.5f), km05 = make_float2(-0.5f, -0.5f);
#pragma unroll
                for (int k = 0; k < KU; ++k) {
                    const float2 dx = __fadd2_rn(X, nx2[k]);
                    const float2 dy = __fadd2_rn(Y, ny2[k]);
                    const float2 dz = __fadd2_rn(Z, nz2[k]);
                    float2 r2 = __ffma2_rn(dx, dx, e2);
                    r2 = __ffma2_rn(dy, dy, r2);
                    r2 = __ffma2_rn(dz, dz, r2);
                    const float2 ri = make_float2(rsqrt_approx(r2.x), rsqrt_approx(r2.y));
                    const float2 qdx = __ffma2_rn(Qxx, dx, __ffma2_rn(Qxy, dy, __fmul2_rn(Qxz, dz)));
                    const float2 qdy = __ffma2_rn(Qxy, dx, __ffma2_rn(Qyy, dy, __fmul2_rn(Qyz, dz)));
                    const float2 qdz = __ffma2_rn(Qxz, dx, __ffma2_rn(Qyz, dy, __fmul2_rn(Qzz, dz)));
                    const float2 sq = __ffma2_rn(qdx, dx, __ffma2_rn(qdy, dy, __ffma2_rn(qdz, dz, C)));
                    const float2 ri2 = __fmul2_rn(ri, ri);
                    const float2 ri3 = __fmul2_rn(ri2, ri);
                    const float2 ri5 = __fmul2_rn(ri3, ri2);
                    const float2 tq = __fmul2_rn(sq, ri5);
                    const float2 A = __ffma2_rn(__fmul2_rn(tq, ri2), km25, __fmul2_rn(M, ri3));
                    b[k][0] = __ffma2_rn(A, dx, __ffma2_rn(ri5, qdx, b[k][0]));
                    b[k][1] = __ffma2_rn(A, dy, __ffma2_rn(ri5, qdy, b[k][1]));
                    b[k][2] = __ffma2_rn(A, dz, __ffma2_rn(ri5, qdz, b[k][2]));
                    b[k][3] = __ffma2_rn(tq, km05, __ffma2_rn(M, ri, b[k][3]));
                }
            }
            since += 2 * (j1 - j0);
        } else {
            const int ps = (h.nn + n_js - 1) / n_js;
            const int j0 = min(h.nn, js * ps);
            const int j1 = min(h.nn, j0 + ps);
#pragma unroll 2
            for (int j = j0; j < j1; ++j) {
                const float4 q0 = T.sp[j][0];
                const float4 qa = T.sp[j][1];
                const float4 qb = T.sp[j][2];
#pragma unroll
                for (int k = 0; k < KU; ++k) {
                    const float dx = q0.x - xih[k];
                    const float dy = q0.y - yih[k];
                    const float dz = q0.z - zih[k];
                    float r2 = fmaf(dx, dx, eps2);
                    r2 = fmaf(dy, dy, r2);
                    r2 = fmaf(dz, dz, r2);
                    const float ri = rsqrt_approx(r2);
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
    };

    for (;;) {
        const int sl = item % kSlots;
        if (!mbar_wait(&s.full[sl], (item / kSlots) & 1u, p.err, p.wait_limit_ns)) return;
        const Hdr h = s.hdr[sl];
        if (h.kind == kItemExit) return;
        if (h.kind == kItemBegin) {
            const WalkDesc wd = p.walks[h.walk];
            rcut2 = (float)wd.rcut2;
            nip = min(kMaxPass, wd.n_i - h.ipass);
            ku = KI;
            if constexpr (KA < KI) {
                if (pass_cost(nip, KA, CT) < pass_cost(nip, KI, CT)) ku = KA;
            }
            S = (nip + ku - 1) / ku;
            n_js = CT / S;
            js = ct / S;
            slot = ct - js * S;
            active = js < n_js;
            gbase = wd.i_begin + h.ipass + slot;
            if constexpr (CO) {
                r_out_walk = sqrt(wd.rcut2);
                rcut2d = wd.rcut2;
                walk_cur = h.walk;
                self_scale = wd.part == 0 ? 1.0 : 0.0;  // parts of a split walk add it once
            }
#pragma unroll
            for (int k = 0; k < KI; ++k) {
                const bool valid = active && k < ku && slot + k * S < nip;
                float hx = 0.f, hy = 0.f, hz = 0.f;
                float4 lo = make_float4(0.f, 0.f, 0.f, 0.f);
                int kb = 0;
                if (valid) {
                    const EpiDev e = p.epi[gbase + k * S];
                    const double dx = e.x - wd.cx, dy = e.y - wd.cy, dz = e.z - wd.cz;
                    hx = (float)dx;
                    hy = (float)dy;
                    hz = (float)dz;
                    lo = make_float4((float)(dx - (double)hx), (float)(dy - (double)hy), (float)(dz - (double)hz),
                                     (float)(e.rs * e.rs));
                    kb = kband_near(fmaxf(fabsf(hx), fmaxf(fabsf(hy), fabsf(hz))), lo.w, eps2);
                }
                if constexpr (PK) {
                    nx2[k] = make_float2(-hx, -hx);
                    ny2[k] = make_float2(-hy, -hy);
                    nz2[k] = make_float2(-hz, -hz);
                } else {
                    xih[k] = hx;
                    yih[k] = hy;
                    zih[k] = hz;
                }
                s.nlo[k][ct] = lo;
                s.nkb[k][ct] = kb;
                if constexpr (CO) {
                    CoRec cr{};
                    cr.id = -1;
                    if (valid) cr = p.epi_co[gbase + k * S];
                    s.co.coi[k][ct] = cr;
                    s.co.dtot[k][ct] = make_float2(0.f, 0.f);
                    s.co.dsoft[k][ct] = make_float2(0.f, 0.f);
                }
                s.cnt[k][ct] = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) s.acc[k][q][ct] = make_float2(0.f, 0.f);
            }
            clear_acc();
            since = 0;
        } else if (h.kind == kItemEP) {
            if (active) {
                if (ku == KI)
                    ep_tile(IntC<KI>{}, h, sl);
                else if constexpr (KA < KI)
                    ep_tile(IntC<KA>{}, h, sl);
                if (since >= kFlush) flush();
            }
        } else if (h.kind == kItemSP) {
            if (active) {
                if (ku == KI)
                    sp_tile(IntC<KI>{}, h, sl);
                else if constexpr (KA < KI)
                    sp_tile(IntC<KA>{}, h, sl);
                if (since >= kFlush) flush();
            }
        } else {  // kItemEnd: reduce the j-slices of the pass and write
            if (active) flush();
            consumers_sync(CT);
            if (active && js == 0) {
                const double G = p.G;
#pragma unroll
                for (int k = 0; k < KI; ++k) {
                    if (!(k < ku && slot + k * S < nip)) continue;
                    double r[4] = {0.0, 0.0, 0.0, 0.0}, rt = 0.0, rs = 0.0;
                    int n = 0;
                    for (int q = 0; q < n_js; ++q) {
                        const int src = q * S + slot;
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            const float2 v = s.acc[k][c][src];
                            r[c] += (double)v.x + (double)v.y;
                        }
                        if constexpr (CO) {
                            const float2 v = s.co.dtot[k][src], w = s.co.dsoft[k][src];
                            rt += (double)v.x + (double)v.y;
                            rs += (double)w.x + (double)w.y;
                        }
                        n += s.cnt[k][src];
                    }
                    const int gi = gbase + k * S;
                    if constexpr (CO) {
                        // self-potential G m / r_out removed (src/hard.hpp:1663-1674)
                        const double self = self_scale * (double)s.co.coi[k][slot].mass / r_out_walk;
                        p.out_accp[gi] = Accp{G * r[0], G * r[1], G * r[2], G * ((r[3] + rt) + self)};
                        p.out_pot_soft[gi] = G * ((r[3] + rs) + self);
                    } else if constexpr (!SR) {
                        p.out_accp[gi] = Accp{G * r[0], G * r[1], G * r[2], G * r[3]};
                    }
                    p.out_nnb[gi] = n;
                }
            }
            consumers_sync(CT);
        }
        mbar_arrive(&s.empty[sl]);
        ++item;
    }
}

template <int CW, int KI, int MINB, bool PK, int MD, int TE, int NS, bool TM>
__global__ __launch_bounds__((CW + 1) * 32, MINB) void ws_kernel(Params p, const __grid_constant__ CUtensorMap tme,
                                                                 const __grid_constant__ CUtensorMap tms) {
    if (p.input_err && *p.input_err) return;  // the inputs failed their check: run nothing
    extern __shared__ __align__(128) unsigned char smem_raw[];
    Smem<CW, KI, PK, TE, NS, MD, TM>& s = *reinterpret_cast<Smem<CW, KI, PK, TE, NS, MD, TM>*>(smem_raw);
    const int tid = threadIdx.x;
    if (tid == 0) {
        for (int i = 0; i < NS; ++i) {
            mbar_init(&s.full[i], 32);
            mbar_init(&s.empty[i], CW * 32);
        }
        if constexpr (TM) {
            mbar_init(&s.tm.bar[0], 1);
            mbar_init(&s.tm.bar[1], 1);
            // make the initialised barriers visible to the TMA (async) proxy
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
    }
    __syncthreads();
    if (tid >= CW * 32)
        producer<CW, KI, PK, MD, TE, NS, TM>(p, s, tid - CW * 32, tme, tms);
    else
        consumer<CW, KI, PK, MD, TE, NS, TM>(p, s, tid);
}

template <int CW, int KI, int MINB, bool PK, int MD = kModeForce, int TE = 128, int NS = 4, bool TM = false>
cudaError_t launch_ws_t(const Params& p, cudaStream_t st, int num_sms, const TensorMaps* tm = nullptr) {
    cudaError_t e = cudaMemsetAsync(p.queue_head, 0, sizeof(int32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(p.n_retest, 0, sizeof(int32_t), st);
    if (e != cudaSuccess) return e;
    if (p.n_walk <= 0) return cudaSuccess;
    static int per_sm = 0;
    const size_t smem = sizeof(Smem<CW, KI, PK, TE, NS, MD, TM>);
    static const CUtensorMap none{};
    if (TM && (!tm || !tm->valid)) return cudaErrorInvalidValue;
    if (per_sm == 0) {
        e = cudaFuncSetAttribute(ws_kernel<CW, KI, MINB, PK, MD, TE, NS, TM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ws_kernel<CW, KI, MINB, PK, MD, TE, NS, TM>, (CW + 1) * 32, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
    }
    int grid = num_sms * per_sm;
    if (grid > p.n_walk) grid = p.n_walk;
    ws_kernel<CW, KI, MINB, PK, MD, TE, NS, TM><<<grid, (CW + 1) * 32, smem, st>>>(p, TM ? tm->epj : none,
                                                                                  TM ? tm->spj : none);
    return cudaGetLastError();
}

__global__ __launch_bounds__(256) void split_j_kernel(const EpjMix* __restrict__ epj, int64_t n_epj,
                                                      EpjF32* __restrict__ epj32, const SpjMix* __restrict__ spj,
                                                      int64_t n_spj, SpjF32* __restrict__ spj32) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_epj; i += stride) {
        const EpjMix e = epj[i];
        EpjF32 o;
        o.xh = (float)e.x;
        o.yh = (float)e.y;
        o.zh = (float)e.z;
        o.xl = (float)(e.x - (double)o.xh);
        o.yl = (float)(e.y - (double)o.yh);
        o.zl = (float)(e.z - (double)o.zh);
        o.m = e.m;
        o.rs2 = e.rs2;
        epj32[i] = o;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_spj; i += stride) {
        const SpjMix e = spj[i];
        SpjF32 o;
        o.xh = (float)e.x;
        o.yh = (float)e.y;
        o.zh = (float)e.z;
        o.xl = (float)(e.x - (double)o.xh);
        o.yl = (float)(e.y - (double)o.yh);
        o.zl = (float)(e.z - (double)o.zh);
        o.m = e.m;
        o.tr = e.tr;
#pragma unroll
        for (int c = 0; c < 6; ++c) o.Q[c] = e.Q[c];
        o.pad[0] = o.pad[1] = 0.f;
        spj32[i] = o;
    }
}

}  // namespace

cudaError_t launch_split_j(const EpjMix* epj, int64_t n_epj, EpjF32* epj32, const SpjMix* spj, int64_t n_spj,
                           SpjF32* spj32, cudaStream_t s) {
    const int64_t n = n_epj > n_spj ? n_epj : n_spj;
    if (n <= 0) return cudaSuccess;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    split_j_kernel<<<(int)blocks, 256, 0, s>>>(epj, n_epj, epj32, spj, n_spj, spj32);
    return cudaGetLastError();
}

// Variants of the warp-specialised kernel: consumer warps, i per consumer
// thread, minimum CTAs per SM, packed FP32x2, and the ring geometry (EP tile
// entries, slots).
cudaError_t launch_ws(const Params& p, cudaStream_t s, int num_sms, int variant, const TensorMaps* tm) {
    switch (variant) {
        case 0: return launch_ws_t<4, 3, 4, false>(p, s, num_sms);
        case 1: return launch_ws_t<4, 3, 4, true, kModeForce, 128, 3, true>(p, s, num_sms, tm);
        case 2: return launch_ws_t<4, 2, 3, true, kModeForce, 256, 4>(p, s, num_sms);
        case 3: return launch_ws_t<4, 3, 4, true, kModeForce, 256, 4>(p, s, num_sms);
        case 4: return launch_ws_t<4, 3, 3, true, kModeForce, 256, 3>(p, s, num_sms);
        case 5: return launch_ws_t<4, 3, 4, true>(p, s, num_sms);
        case 6: return launch_ws_t<4, 3, 3, true, kModeForce, 256, 4>(p, s, num_sms);
        case 7: return launch_ws_t<4, 3, 3, true, kModeForce, 128, 6>(p, s, num_sms);
        default: return cudaErrorInvalidValue;
    }
}

bool ws_variant_uses_tma(int variant) { return variant == 1; }

cudaError_t launch_ws_search(const Params& p, cudaStream_t s, int num_sms) {
    return launch_ws_t<4, 3, 4, false, kModeSearch>(p, s, num_sms);
}

// Packed far and SP tiles, 128-entry EP tiles, 2 CTAs per SM: the fastest of
// the changeover configurations timed on the 1M binary workload (26.7 ms,
// against 30.3 ms for scalar 64-entry tiles at 3 CTAs per SM).
cudaError_t launch_ws_changeover(const Params& p, cudaStream_t s, int num_sms) {
    return launch_ws_t<4, 3, 2, true, kModeChangeover, 128, 4>(p, s, num_sms);
}

}  // namespace pgf
