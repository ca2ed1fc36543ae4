// Device data layout and kernel interfaces of the soft-force library.
//
// HBM layout (one copy per process, grown on demand, never shrunk):
//   EpjMix[n_epj_tot]    32 B: FP64 position, FP32 mass, FP32 r_search^2
//   epj_m64[n_epj_tot]    8 B: FP64 mass       (plain FP64 kernel)
//   epj_rs64[n_epj_tot]   8 B: FP64 r_search   (plain FP64 kernel, exact re-tests)
//   SpjMix[n_spj_tot]    64 B: FP64 position, FP32 mass, FP32 traceless
//                              quadrupole Q = 3q - tr(q) I and tr(q)
//   SpjQ64[n_spj_tot]    64 B: FP64 mass and raw quadrupole (plain FP64 kernel)
//   EpjF32[n_epj_tot]    32 B: position as an FP32 (hi, lo) pair, FP32 mass
//                              and r_search^2 (warp-specialised kernels)
//   SpjF32[n_spj_tot]    64 B: position as an FP32 (hi, lo) pair, FP32 mass,
//                              traceless quadrupole and tr(q)
//   EpiDev[ni_tot]       32 B: FP64 position and r_search
//   id_epj / id_spj      int32 per list entry, walks concatenated
//   WalkDesc[n_walk]     96 B: list offsets, walk centre (FP64), box
//                              half-extents, largest i r_search, r_out^2
//   order[n_walk]        walks sorted by descending work (the work queue)
//   out_accp[ni_tot]     Accp (32 B): acc.xyz, pot (G applied)
//   out_nnb[ni_tot]      int32 neighbour count
// The j arrays of a 1.5M-particle problem (about 50 MB EPJ + 18 MB SPJ for the
// mixed kernel) stay resident in the 129 MB L2 while the id lists stream from
// HBM once per force evaluation.
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace pgf {

struct __align__(32) EpjMix {
    double x, y, z;
    float m;
    float rs2;  // (float)(r_search * r_search), the square taken in FP64
};
static_assert(sizeof(EpjMix) == 32, "EpjMix layout");

struct __align__(32) SpjMix {
    double x, y, z;
    float m;
    float pad0;
    float Q[6];  // traceless 3q - tr(q) I: xx, yy, zz, xy, xz, yz
    float tr;    // tr(q)
    float pad1;
};
static_assert(sizeof(SpjMix) == 64, "SpjMix layout");

// Positions split into FP32 hi = fl(x) and lo = fl(x - hi), so hi + lo holds x
// to about 2^-48 |x|.  Built on the device from EpjMix / SpjMix; they let the
// warp-specialised kernels form walk-relative coordinates in FP32 arithmetic
// (the FP64 pipe of GB300 runs at 1/64 of the FP32 rate).
struct __align__(32) EpjF32 {
    float xh, yh, zh, m;
    float xl, yl, zl, rs2;
};
static_assert(sizeof(EpjF32) == 32, "EpjF32 layout");

struct __align__(32) SpjF32 {
    float xh, yh, zh, m;
    float xl, yl, zl, tr;
    float Q[6];  // traceless 3q - tr(q) I
    float pad[2];
};
static_assert(sizeof(SpjF32) == 64, "SpjF32 layout");

// Acceleration of one EPJ as an FP32 (hi, lo) pair (KDKDK_4TH gradient mode):
// differences a_j - a_i are formed from both halves, accurate to an ulp of
// the difference itself.
struct __align__(32) AccF32 {
    float xh, yh, zh, pad0;
    float xl, yl, zl, pad1;
};
static_assert(sizeof(AccF32) == 32, "AccF32 layout");

// Changeover data of one particle for the fused changeover mode: the
// ChangeOver members of src/changeover.hpp:8-14 (r_in, r_out, norm =
// 1/(r_out - r_in), coff = (r_out - r_in)/(r_out + r_in), pot_off =
// (1 + coff)/r_out), computed in FP64 and rounded; the particle id; and a mass:
// for EPJ the mass its neighbours' potentials use (m for singles, mass_backup
// for members, 0 otherwise), for EPI the mass of its self-potential term.
struct __align__(32) CoRec {
    float r_in, r_out, norm, coff;
    float pot_off, mass;
    int64_t id;
};
static_assert(sizeof(CoRec) == 32, "CoRec layout");

struct __align__(16) SpjQ64 {
    double m;
    double q[6];  // raw second moment: xx, yy, zz, xy, xz, yz (zero for monopoles)
    double pad;
};
static_assert(sizeof(SpjQ64) == 64, "SpjQ64 layout");

struct __align__(32) EpiDev {
    double x, y, z, rs;
};
static_assert(sizeof(EpiDev) == 32, "EpiDev layout");

struct __align__(32) WalkDesc {
    int64_t epj_begin;  // offset of the walk's EPJ ids in id_epj
    int64_t spj_begin;  // offset of the walk's SPJ ids in id_spj
    int32_t i_begin;    // first EPI row of the walk
    int32_t n_i;
    int32_t n_epj;
    int32_t n_spj;
    double cx, cy, cz;  // walk centre: centre of the EPI bounding box
    double rcut2;       // r_out^2 of the walk
    float hx, hy, hz;   // EPI box half-extents, rounded up
    float rs_max;       // largest r_search of the walk's EPI, rounded up
    int32_t part;       // 0, or k >= 1 for part k of a split walk (adds no per-i terms)
    float pad[3];
};
static_assert(sizeof(WalkDesc) == 96, "WalkDesc layout");

// Result of one i-particle: acceleration and potential with G applied.
struct __align__(32) Accp {
    double x, y, z, w;
};
static_assert(sizeof(Accp) == 32, "Accp layout");

// An (i, EPJ tile) whose FP32 neighbour test came within rounding distance of
// r_search for some pair: the retest kernel recounts the tile in FP64.
struct Retest {
    int64_t j_begin;  // offset in id_epj
    int32_t i;        // EPI row
    int32_t n;        // number of list entries
    int32_t walk;     // walk (descriptor index) of the i-particle
    int32_t pad;
};

struct Params {
    const EpiDev* epi;
    const EpjMix* epj;
    const double* epj_m64;
    const double* epj_rs64;
    const SpjMix* spj;
    const SpjQ64* spj_q64;
    const EpjF32* epj32;
    const SpjF32* spj32;
    const CoRec* epj_co;   // fused changeover mode only (else null)
    const CoRec* epi_co;
    double* out_pot_soft;  // fused changeover mode: soft potential (G applied)
    const AccF32* epj_acc32;  // gradient mode: EPJ accelerations (hi, lo)
    const Accp* epi_acc64;    // gradient mode: EPI accelerations (x, y, z; w unused)
    Accp* out_acorr;          // gradient mode: acorr (no G; w unused)
    const int32_t* id_epj;
    const int32_t* id_spj;
    const WalkDesc* walks;
    const int32_t* order;
    int32_t n_walk;
    int32_t pad0;
    double eps2;
    double G;
    Accp* out_accp;
    int32_t* out_nnb;
    // scratch
    int32_t* queue_head;   // work-queue cursor, zeroed before each launch
    Retest* retest;        // FP64 re-test records
    int32_t* n_retest;     // number of records pushed (may exceed capacity)
    int32_t retest_cap;
    int32_t pad1;
    int32_t* err;          // device error word (0 = ok)
    int32_t* retest_total; // records re-tested since the host last read it (optional)
    // Walk count written by an earlier kernel on the same stream (the device
    // list builder), or null: the kernels then run min(*n_walk_dev, n_walk)
    // walks, n_walk being the capacity of walks and order.
    const int32_t* n_walk_dev;
    // Limit of every bounded wait in the warp-specialised kernels (0: 1 s).
    uint64_t wait_limit_ns;
    // Test hook: > 0 makes their producer stop after that many ring items.
    int32_t stall_after_items;
    int32_t gr_compensated;  // gradient pass: r^2 and 1/r of far pairs to about 2^-40 (pgf_set_gradient_accuracy)
    // Result of the device-side check of a host-direct dispatch's ids, or
    // null: when it is non-zero the force kernels run nothing.
    const int32_t* input_err;
};

// Number of walks of this launch.
__device__ __forceinline__ int walk_count(const Params& p) {
    return p.n_walk_dev ? min(*p.n_walk_dev, p.n_walk) : p.n_walk;
}

// Exact FP64 neighbour test of one pair, in the oracle's evaluation order
// (src/force_gpu_cuda.cu:62-64 semantics, src/soft_force.hpp:58-64 order):
// r2 = ((dx*dx) + (dy*dy)) + (dz*dz); (r2 + eps2) < max(rs_i, rs_j)^2.
__device__ __forceinline__ int exact_neighbour(double xi, double yi, double zi, double rsi, double xj,
                                               double yj, double zj, double rsj, double eps2) {
    const double dx = __dsub_rn(xi, xj);
    const double dy = __dsub_rn(yi, yj);
    const double dz = __dsub_rn(zi, zj);
    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
    const double rs = rsi > rsj ? rsi : rsj;
    return __dadd_rn(r2, eps2) < __dmul_rn(rs, rs) ? 1 : 0;
}

// FP64 difference between the changeover pair terms and the linear-cutoff
// pair terms of one neighbour pair (the fused mode's correction for pairs
// whose neighbour status only the FP64 re-test decides): acceleration x, y,
// z, pot_tot and pot_soft, without G.  Same formulas as the FP32 pair path.
__device__ __forceinline__ void co_pair_diff(const EpiDev& ei, const CoRec& ci, const EpjMix& ej, float mj, const CoRec& cj,
                                    double eps2, double rcut2, double out[5]) {
    const double dx = ej.x - ei.x, dy = ej.y - ei.y, dz = ej.z - ei.z;
    const double r2 = dx * dx + dy * dy + dz * dz + eps2;
    const double r = sqrt(r2), ri = 1.0 / r;
    const double rimax = 1.0 / sqrt(r2 > rcut2 ? r2 : rcut2);
    const CoRec& c = ci.r_out > cj.r_out ? ci : cj;
    const double x = (r - (double)c.r_in) * (double)c.norm;
    const double xa = x < 0.0 ? 0.0 : (x > 1.0 ? 1.0 : x);
    const double x_1 = xa - 1.0, x_2 = x_1 * x_1, xa2 = xa * xa;
    const double wacc = (x_2 * x_2) * (1.0 + 4.0 * xa + 10.0 * xa2 + 20.0 * xa2 * xa + 35.0 * (double)c.coff * xa2 * xa2);
    double wpot = 1.0;
    if (x >= 1.0) {
        wpot = (double)c.pot_off * r;
    } else if (x > 0.0) {
        const double x2 = x * x, x3 = x2 * x;
        wpot = 1.0 - (double)c.coff * (x2 * x3) * (5.0 * x3 - 20.0 * x2 + 28.0 * x - 14.0);
    }
    const double f = (double)mj * ((1.0 - wacc) * ri * ri * ri - rimax * rimax * rimax);
    out[0] = f * dx;
    out[1] = f * dy;
    out[2] = f * dz;
    const double meff = (double)cj.mass;
    out[3] = -meff * ri + (double)mj * rimax;
    out[4] = -meff * (1.0 - wpot) * ri + (double)mj * rimax;
}

// A walk whose list was split into n_parts parts (small dispatches, to spread
// the largest walks over several CTAs): part 0 writes the walk's own EPI rows
// from row0, part k >= 1 a copy of them from rows1 + (k - 1) n_i.
struct SplitRec {
    int32_t row0, rows1, n_i, n_parts;
};

// ---- Host-direct data movement (pgf_hostdirect.cu) ----
// The GPU reads the caller's records in host memory through the host page
// tables and writes results into them; these tables and arguments describe
// where.

// One walk of a host-direct dispatch, in layout order.
struct WalkSrc {
    const char* epi;        // the caller's EPI records of the walk
    const int32_t* id_epj;  // the caller's id lists of the walk
    const int32_t* id_spj;
    int64_t i_off, e_off, s_off;  // first EPI row and list entries in the device arrays
    int64_t rows1;          // split walks: first EPI row of part 1's copy
    double rcut2;           // r_out^2 of the walk
    int32_t n_i, n_epj, n_spj;
    int32_t walk;           // the caller's walk index (error reports)
    int32_t parts;          // 1, or the parts of a split walk
    int32_t desc1;          // split walks: descriptor index of part 1
    int32_t split;          // split walks: index of its SplitRec
    int32_t pad;
};

// Where retrieve writes walk k's results.
struct ForceDst {
    char* base;   // the caller's Force records of the walk
    int64_t row;  // first result row of the walk
    int32_t n;
    int32_t pad;
};

struct HdSendArgs {
    const char* epj;
    int64_t n_epj;
    size_t epj_size, epj_off_mass, epj_off_pos, epj_off_rs;
    const char* spj;
    int64_t n_spj;
    size_t spj_size, spj_off_mass, spj_off_pos, spj_off_quad;
    int spj_has_quad;
    // fused changeover mode (out_epj_co non-null)
    size_t co_epj_off_id, co_epj_off_r_in, co_epj_off_r_out, co_epj_off_mass_backup, co_epj_off_status;
    // gradient mode (out_epj_acc32 non-null)
    size_t gr_epj_off_acc;
    EpjMix* out_epj;
    double* out_epj_m64;
    double* out_epj_rs64;
    EpjF32* out_epj32;
    CoRec* out_epj_co;
    AccF32* out_epj_acc32;
    SpjMix* out_spj;
    SpjQ64* out_spj_q64;
    SpjF32* out_spj32;
};

struct HdWalkArgs {
    const WalkSrc* src;         // pinned host table, read in place
    int n_walk;
    int n_desc;                 // work-queue entries (walks and parts)
    const int32_t* order_src;   // pinned host work-queue order, copied to order_dst
    int32_t* order_dst;
    SplitRec* out_splits;       // split walks' records (combine kernel)
    size_t epi_size, epi_off_pos, epi_off_rs;
    size_t gr_epi_off_acc;  // gradient mode (out_epi_acc non-null)
    size_t co_epi_off_id, co_epi_off_r_in, co_epi_off_r_out, co_epi_off_self_mass;  // changeover (out_epi_co)
    int64_t n_epj_tot, n_spj_tot;
    EpiDev* out_epi;
    Accp* out_epi_acc;
    CoRec* out_epi_co;
    int32_t* out_id_epj;
    int32_t* out_id_spj;
    WalkDesc* out_walks;
    // [0] set when an id is out of range, [1] the largest such caller walk
    // index, [2] finished CTAs, [3] the outcome the force kernels read.  The
    // last CTA moves [0], [1] into err_host[0], [1] (pinned) and [3], and
    // clears [0..2] for the next dispatch.
    int32_t* err;
    int32_t* err_host;
};

struct HdScatterArgs {
    const ForceDst* dst;
    int n_walk;
    int counts_only;  // neighbour search: n_ngb only
    size_t size, off_acc, off_pot, off_nnb;
    int nnb_bytes;
    int pad;
    size_t off_pot_soft, off_acorr;
    const Accp* accp;
    const int32_t* nnb;
    const double* pot_soft;  // changeover mode, else null
    const Accp* acorr;       // gradient mode, else null
    // Status words of the evaluation (the device error word and the re-test
    // total at [2], [3]): copied to flags_host and cleared by the kernel.
    int32_t* flags_dev;
    int32_t* flags_host;
};

cudaError_t launch_gather_j(const HdSendArgs& a, int num_sms, cudaStream_t s);
cudaError_t launch_gather_walks(const HdWalkArgs& a, int num_sms, cudaStream_t s);
cudaError_t launch_scatter_results(const HdScatterArgs& a, int num_sms, cudaStream_t s);

// Launchers (stream-ordered, asynchronous).
cudaError_t launch_fp64(const Params& p, cudaStream_t s, int num_sms);
cudaError_t launch_mixed(const Params& p, cudaStream_t s, int num_sms);
cudaError_t launch_retest(const Params& p, cudaStream_t s, int num_sms);
// Adds the results of every split walk's parts into its own rows, parts in
// order (deterministic).
// pot_soft and acorr (optional) are the changeover and gradient modes' outputs.
cudaError_t launch_combine_parts(const SplitRec* recs, int n_recs, Accp* accp, int32_t* nnb, double* pot_soft,
                                 Accp* acorr, cudaStream_t s);
// Copies every split walk's EPI rows (and its changeover / gradient records,
// when given) from row0 to the rows of parts 1 .. n_parts-1.
cudaError_t launch_split_rows(const SplitRec* recs, int n_recs, EpiDev* epi, CoRec* co, Accp* acc, cudaStream_t s);
// Builds the (hi, lo) FP32 copies of the EPJ / SPJ arrays.
cudaError_t launch_split_j(const EpjMix* epj, int64_t n_epj, EpjF32* epj32, const SpjMix* spj, int64_t n_spj,
                           SpjF32* spj32, cudaStream_t s);
// Warp-specialised kernel, variants 0..kNumWsVariants-1 (see pgf_kernels_ws.cu).
constexpr int kNumWsVariants = 8;
// TMA descriptors of the (hi, lo) EPJ and SPJ arrays (rows of 32 and 64
// bytes, boxes one row high), rebuilt at every send.
struct TensorMaps {
    CUtensorMap epj;
    CUtensorMap spj;
    bool valid = false;
};
cudaError_t launch_ws(const Params& p, cudaStream_t s, int num_sms, int variant, const TensorMaps* tm);
// Whether warp-specialised variant v stages its tiles with TMA (needs TensorMaps).
bool ws_variant_uses_tma(int variant);
// Neighbour search (counts only, SPJ lists ignored) with the warp-specialised kernel.
cudaError_t launch_ws_search(const Params& p, cudaStream_t s, int num_sms);
// Soft force with the changeover correction of neighbours fused in.
cudaError_t launch_ws_changeover(const Params& p, cudaStream_t s, int num_sms);
// KDKDK_4TH gradient-correction pass (pgf_kernels_gradient.cu).
cudaError_t launch_gradient(const Params& p, cudaStream_t s, int num_sms);

}  // namespace pgf
