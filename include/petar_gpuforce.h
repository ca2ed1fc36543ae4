/* C ABI of the GB300 soft-force kernels for PeTar.
 *
 * These entry points replace PeTar's CUDA soft-force functor pair:
 *   CalcForceWithLinearCutoffCUDAMultiWalk  src/force_gpu_cuda.hpp:103-133,
 *                                           src/force_gpu_cuda.cu:535-700
 *   CalcForceWithLinearCutoffCUDA           src/force_gpu_cuda.hpp:137-162,
 *                                           src/force_gpu_cuda.cu:704-827
 *   RetrieveForceCUDA                       src/force_gpu_cuda.hpp:165-168,
 *                                           src/force_gpu_cuda.cu:831-880
 * and their profiling counters (GPUProfile / GPUCounter,
 * src/force_gpu_cuda.hpp:6-93).
 *
 * Particle arrays are passed as the caller's own records (FDPS's EPISoft,
 * EPJSoft, SPJSoft and ForceSoft in PeTar) together with a layout that gives
 * the record size and the byte offsets of the fields the kernels read or
 * write.  Positions are three consecutive doubles (FDPS F64vec), the
 * quadrupole is six consecutive doubles in FDPS MatrixSym order
 * (xx, yy, zz, xy, xz, yz).  The header include/petar_gpuforce.hpp wraps these
 * calls in functors with the reference signatures.
 *
 * All functions return PGF_OK (0) or a PGF_ERR_* code; pgf_last_error() gives
 * a message for the last failure.  The reference returned 0 and asserted; the
 * C++ wrapper keeps that by aborting on a non-zero code.
 *
 * Threading: like the reference, one process drives one device through
 * file-scope state; calls are not re-entrant.
 */
#ifndef PETAR_GPUFORCE_H
#define PETAR_GPUFORCE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    PGF_OK = 0,
    PGF_ERR_ARG = 1,        /* invalid argument (null pointer, negative size, bad tag) */
    PGF_ERR_NO_DEVICE = 2,  /* no CUDA device visible */
    PGF_ERR_CUDA = 3,       /* a CUDA runtime call failed */
    PGF_ERR_STATE = 4,      /* call out of sequence (e.g. retrieve without dispatch) */
    PGF_ERR_CAPACITY = 5,   /* a size exceeds what the kernels index (2^31-1 rows) */
    PGF_ERR_DEVICE = 6      /* the kernels reported an error flag (bounded wait expired) */
};

/* Kernel selection for pgf_set_precision. */
enum {
    PGF_PRECISION_MIXED = 0, /* FP64 walk-relative coordinates, FP32 pair arithmetic,
                                FP64 cross-tile sums, exact neighbour counts (default) */
    PGF_PRECISION_FP64 = 1   /* plain FP64 throughout */
};

/* What an index dispatch computes (pgf_set_mode). */
enum {
    PGF_MODE_FORCE = 0,           /* soft force: acc, pot and n_ngb (default) */
    PGF_MODE_NEIGHBOR_SEARCH = 1, /* n_ngb only, as SearchNeighborEpEpNoSimd
                                     (src/soft_force.hpp:11-34): r^2 < max(rs_i, rs_j)^2
                                     without softening; SPJ lists are ignored */
    PGF_MODE_FORCE_CHANGEOVER = 2, /* soft force with the changeover correction of
                                     neighbours fused in (see pgf_set_changeover_layout) */
    PGF_MODE_GRADIENT = 3         /* KDKDK_4TH gradient-correction pass (see
                                     pgf_set_gradient_layout) */
};

/* KDKDK_4TH gradient-correction pass (src/petar.hpp:1123-1140), run on the CPU
 * by the reference: per i, CalcCorrectEpEpWithLinearCutoffNoSimd
 * (src/soft_force.hpp:89-122) over the EPJ list and the quadrupole force over
 * the SPJ list, into one cleared ForceSoft:
 *   acorr = 2 sum_j -m_j / r^3 (da - 3 (dr.da) / r^2 dr)  (no G; dr = x_i - x_j,
 *           da = a_i - a_j, r^2 = max(|dr|^2 + eps^2, r_out^2)),
 *   acc = a_i + G acc_sp, pot = G pot_sp, n_ngb = 0.
 * The EPI and EPJ records carry the particle's acceleration (EPISoft::acc,
 * EPJSoft::acc under KDKDK_4TH) and the Force record acorr, at these byte
 * offsets (three F64 each).  Set the layout before the send. */
typedef struct pgf_gradient_layout {
    size_t epi_off_acc;
    size_t epj_off_acc;
    size_t force_off_acorr;
} pgf_gradient_layout;

/* Sets (or with NULL clears) the layout of the gradient mode.  No
 * counterpart in the reference, whose pass runs on the CPU. */
int pgf_set_gradient_layout(const pgf_gradient_layout *layout);

/* Accuracy of the gradient pass's pairs beyond r_out: 1 (default)
 * compensated, with r^2 and 1/r carried to about 2^-40 (exact squares,
 * error-free sums and a residual-corrected rsqrt) and the acorr partial
 * sums flushed every 8 j pairs; 0 plain FP32, about 1.3 times faster.  The
 * sum over j of the gradient correction cancels 100-200-fold for some
 * members of close binaries, where FP32 rounding of r^2 and 1/r leaves
 * p99.9 errors up to about 1.6e-5; the compensated mode stays under 1e-5.
 * Pairs inside r_out run in double-float in both modes. */
int pgf_set_gradient_accuracy(int mode);

/* Fused changeover mode.  PeTar corrects the soft force on the CPU after the
 * kernel: for every tree neighbour j of i, calcAccPotShortWithLinearCutoff
 * (src/hard.hpp:1404-1480) replaces the linear-cutoff pair term by the
 * changeover force G m_j (1 - W_acc(r)) / r^3 (W of the pair's larger
 * r_out, src/changeover.hpp:294-334, 364-375) and splits the potential into
 * pot_tot and pot_soft by j's artificial-particle status; the particle's own
 * G m / r_out self-term is removed (src/hard.hpp:1663-1674).  In this mode
 * the kernel evaluates the corrected result directly.  Neighbours are the
 * pairs the neighbour count counts (|dx|^2 + eps^2 < max(rs_i, rs_j)^2, the
 * tree search's test when eps = 0), the particle itself (same id) excluded.
 * The caller's records carry the extra fields at these byte offsets: ids are
 * 8-byte integers, everything else F64.  Set the layout before the send
 * (send_flag) so that the EPJ changeover data is packed with the EPJ array;
 * retrieve writes the total potential to pot and the soft one to pot_soft. */
typedef struct pgf_changeover_layout {
    size_t epi_off_id;          /* EPI: particle id */
    size_t epi_off_r_in;        /* EPI: changeover r_in */
    size_t epi_off_r_out;       /* EPI: changeover r_out */
    size_t epi_off_self_mass;   /* EPI: mass of the self-potential term to remove (0: none) */
    size_t epj_off_id;          /* EPJ: particle id */
    size_t epj_off_r_in;        /* EPJ: changeover r_in (EPJSoft::r_in) */
    size_t epj_off_r_out;       /* EPJ: changeover r_out (EPJSoft::r_out) */
    size_t epj_off_mass_backup; /* EPJ: group_data.artificial mass_backup */
    size_t epj_off_status;      /* EPJ: group_data.artificial status */
    size_t force_off_pot_soft;  /* Force: F64 soft potential (written) */
} pgf_changeover_layout;

/* Sets (or with NULL clears) the changeover layout used by the send and by
 * dispatches in PGF_MODE_FORCE_CHANGEOVER.  No counterpart in the reference,
 * whose correction runs on the CPU. */
int pgf_set_changeover_layout(const pgf_changeover_layout *layout);

/* Record layouts (sizes and byte offsets). */
typedef struct pgf_epi_layout {
    size_t size;         /* sizeof(EPISoft) */
    size_t off_pos;      /* F64vec pos */
    size_t off_r_search; /* F64 r_search */
} pgf_epi_layout;

typedef struct pgf_epj_layout {
    size_t size;         /* sizeof(EPJSoft) */
    size_t off_mass;     /* F64 mass */
    size_t off_pos;      /* F64vec pos */
    size_t off_r_search; /* F64 r_search */
} pgf_epj_layout;

typedef struct pgf_spj_layout {
    size_t size;         /* sizeof(SPJSoft) */
    size_t off_mass;     /* F64 mass */
    size_t off_pos;      /* F64vec pos */
    size_t off_quad;     /* F64mat quad (xx, yy, zz, xy, xz, yz); ignored when has_quad == 0 */
    int has_quad;        /* 0: monopole superparticles (SPJMonopoleInAndOut) */
} pgf_spj_layout;

typedef struct pgf_force_layout {
    size_t size;         /* sizeof(ForceSoft) */
    size_t off_acc;      /* F64vec acc (overwritten) */
    size_t off_pot;      /* F64 pot (overwritten) */
    size_t off_n_ngb;    /* integer n_ngb (overwritten) */
    int n_ngb_bytes;     /* 4 or 8 */
} pgf_force_layout;

/* Timings (seconds, accumulated since the last pgf_clear_profile) and
 * counters, mirroring GPUProfile / GPUCounter (src/force_gpu_cuda.hpp:6-93). */
typedef struct pgf_profile {
    double copy;         /* host packing and unpacking */
    double send;         /* host-to-device copies */
    double recv;         /* device-to-host copies */
    double calc;         /* kernels, all of them */
    double calc_main;    /* the interaction kernel alone */
    double last_calc;    /* kernels of the most recent dispatch */
    double last_calc_main;
    int64_t n_walk, n_epi, n_epj, n_spj, n_call;
    int64_t n_retest;    /* pair ranges re-tested in FP64 for exact neighbour counts */
} pgf_profile;

/* CalcForceWithLinearCutoffCUDAMultiWalk constructor / initialize()
 * (src/force_gpu_cuda.hpp:109-118).  Selects device rank % device_count on
 * the first call, as src/force_gpu_cuda.cu:549-553 does. */
int pgf_initialize(int rank, double eps2, double rcut2, double G);

/* Chooses the kernel used by later dispatches (PGF_PRECISION_*). */
int pgf_set_precision(int precision);

/* Selects what later dispatches compute (PGF_MODE_*).  Each tag keeps the
 * mode of its dispatch; retrieve of a neighbour-search dispatch overwrites
 * n_ngb only and leaves acc and pot as they are.  The GPU counterpart of the
 * reference's CPU search functor SearchNeighborEpEpNoSimd
 * (src/soft_force.hpp:11-34); counts are exact as in the force mode. */
int pgf_set_mode(int mode);

/* Mixed-precision kernel variants: 0 is the CTA-synchronous tiled kernel;
 * 1..PGF_NUM_KERNEL_VARIANTS-1 are warp-specialised producer/consumer kernels
 * with different consumer-warp counts, i-particles per thread and scalar or
 * packed FP32x2 arithmetic.  The choice applies to later dispatches. */
#define PGF_NUM_KERNEL_VARIANTS 9
/* The variant used until one is chosen: the warp-specialised kernel with
 * 256-entry EP tiles, the fastest on the 1M binary Plummer and the King 4M
 * workloads on GB300.  pgf_autotune picks per workload. */
#define PGF_DEFAULT_KERNEL_VARIANT 7
int pgf_set_kernel_variant(int variant);
int pgf_get_kernel_variant(int *variant);

/* Index dispatches run as a pipeline of up to 8 stages over contiguous walk
 * ranges (host packing, copies and kernels of successive stages overlap).
 * 0 (default) picks the stage count from the id-list size, 1 disables the
 * pipeline, 2..8 force that many stages (dispatches of fewer than 8 walks per
 * stage use one).  Results do not depend on the stage count. */
int pgf_set_dispatch_stages(int stages);

/* Walk splitting in single-launch dispatches (1, the default, or 0 = off).
 * When a dispatch has few walks for the GPU's CTAs, each walk costing more
 * than a sixteenth of one SM's even share runs as up to 16 parts over slices
 * of its EPJ and SPJ lists, and the parts are added in a fixed order; results then differ
 * from an unsplit launch by FP32 summation order only (counts are exact).
 * All modes; no counterpart in the reference. */
int pgf_set_walk_split(int enable);

/* Split unit of walk splitting: a walk is split when it costs more than
 * 1/div of one SM's even share of the dispatch (default 16; 1..256).
 * pgf_autotune_dispatch sets it too.  Results are as for pgf_set_walk_split. */
int pgf_set_walk_split_unit(int div);

/* Limit of every bounded wait inside the warp-specialised kernels, in
 * nanoseconds of the GPU's global timer (0 restores the default, 1 s).  A
 * wait that runs out sets the device error word and its warp returns, so the
 * kernel ends and the next retrieve reports PGF_ERR_DEVICE instead of the
 * launch hanging.  No counterpart in the reference, whose kernels do not wait. */
int pgf_set_wait_limit_ns(uint64_t limit_ns);
/* Test hook for the path above: with items > 0 the producer warp of the
 * warp-specialised kernels stops publishing ring items after that many, so
 * that the consumers' waits run out (no fault, no trap; every warp returns).
 * 0 (the default) turns it off.  For failure-detection tests only. */
int pgf_test_stall_producer(int items);

/* Host-direct data movement (1, the default, or 0 = off).  On GB300 the GPU
 * reads ordinary (pageable) host memory coherently through the host page
 * tables over NVLink-C2C.  When the device reports that
 * (cudaDevAttrPageableMemoryAccess), the send phase and single-launch walk
 * dispatches read the caller's records and id lists in place with a gather
 * kernel, and retrieve of a single-launch dispatch writes results into the
 * caller's Force records with a scatter kernel, instead of packing on the
 * host into pinned staging and copying.  Pipelined dispatches keep the host
 * packing and unpacking of their walks, which overlap the kernels of other
 * stages on the copy engines and host cores.  The device arrays, and so the results, are bit-identical either
 * way; ids are still checked before any force kernel runs.  The caller's
 * arrays must stay valid and unchanged for the duration of each call, as the
 * reference requires.  No counterpart in the reference, whose host code
 * packs on the CPU (src/force_gpu_cuda.cu:577-699, 866-875). */
int pgf_set_host_direct(int enable);
/* *active = 1 when later calls move data host-direct (enabled and supported). */
int pgf_get_host_direct(int *active);

/* Autotuner: times every kernel variant `repeats` times on the data of the
 * tag's last index dispatch (already on the device), keeps the fastest for
 * later dispatches and reports it and its mean main-kernel time.  The results
 * of the tag are those of the last variant run; retrieve after a recompute. */
int pgf_autotune(int tag, int repeats, int *best_variant, double *best_ms);

/* Autotuner for the dispatch itself: runs the caller's walk dispatch and
 * retrieve (the arguments of pgf_dispatch_index's walk phase and of
 * pgf_retrieve; the j arrays must have been sent) for each candidate, best of
 * `repeats` timed runs after a warm-up, and keeps the fastest for later
 * dispatches.  Candidates: pipeline stage counts 1, 2, 4 and 8 (how many
 * launches a dispatch is cut into, each overlapping the next stage's packing
 * and copies), and for single launches the walk-split unit (a sixteenth of
 * one SM's even share by default; 4, 8 and 32 also tried).  The force records
 * hold the last run's results.  The reference fixes its walks per launch at
 * compile time (N_WALK_LIMIT, src/force_gpu_cuda.cu:12-17) and PeTar its
 * n_walk_limit (src/petar.hpp:888). */
int pgf_autotune_dispatch(int tag, int n_walk, const void *const *epi, const int *n_epi,
                          const pgf_epi_layout *epi_layout, const int *const *id_epj, const int *n_epj,
                          const int *const *id_spj, const int *n_spj, void *const *force,
                          const pgf_force_layout *force_layout, int repeats, int *best_stages, int *best_split,
                          double *best_ms);

/* Launch on the caller's CUDA stream (a cudaStream_t passed as void*);
 * NULL restores the library's own stream. */
int pgf_set_stream(void *cuda_stream);

/* CalcForceWithLinearCutoffCUDAMultiWalk::operator()
 * (src/force_gpu_cuda.hpp:120-132, src/force_gpu_cuda.cu:535-700).
 * send_flag != 0: copies the shared EPJ/SPJ arrays to the device and returns.
 * send_flag == 0: packs the walks' EPI and id lists, copies them and launches
 * the kernels for all n_walk walks; returns without waiting for the kernels.
 * Unused arguments may be NULL for each phase. */
int pgf_dispatch_index(int tag, int n_walk,
                       const void *const *epi, const int *n_epi, const pgf_epi_layout *epi_layout,
                       const int *const *id_epj, const int *n_epj,
                       const int *const *id_spj, const int *n_spj,
                       const void *epj, int n_epj_tot, const pgf_epj_layout *epj_layout,
                       const void *spj, int n_spj_tot, const pgf_spj_layout *spj_layout,
                       int send_flag);

/* CalcForceWithLinearCutoffCUDA::operator() (src/force_gpu_cuda.hpp:154-161,
 * src/force_gpu_cuda.cu:704-827): per-walk EPJ/SPJ arrays, no id lists. */
int pgf_dispatch(int tag, int n_walk,
                 const void *const *epi, const int *n_epi, const pgf_epi_layout *epi_layout,
                 const void *const *epj, const int *n_epj, const pgf_epj_layout *epj_layout,
                 const void *const *spj, const int *n_spj, const pgf_spj_layout *spj_layout);

/* RetrieveForceCUDA (src/force_gpu_cuda.hpp:165-168,
 * src/force_gpu_cuda.cu:831-880): waits for the dispatch of this tag and
 * overwrites acc, pot and n_ngb of force[w][0..ni[w]). */
int pgf_retrieve(int tag, int n_walk, const int *ni, void *const *force,
                 const pgf_force_layout *force_layout);

/* Per-walk r_out^2 for the next index dispatch of independent clusters in one
 * launch (NULL or n_walk == 0 clears it).  Extends the reference, whose r_out
 * is one functor constant (src/petar.hpp:889-891). */
int pgf_set_walk_rcut2(const double *walk_rcut2, int n_walk);

/* Re-runs the kernels of the last index dispatch of this tag on the data
 * already on the device (no host packing, no copies); returns immediately. */
int pgf_recompute(int tag);

/* Waits for the kernels of the tag's last dispatch or recompute and adds
 * their times to the profile, without copying results back. */
int pgf_wait(int tag);

/* Profiling counters (GPUProfile / GPUCounter). */
int pgf_get_profile(pgf_profile *out);
int pgf_clear_profile(void);

/* Message for the last failure ("" when none). */
const char *pgf_last_error(void);

/* ---- Allocation-free variant (no counterpart in the reference) ----
 *
 * For callers that cannot let a library allocate device memory: codes that
 * carve all device memory out of one arena they size at start-up, or loops
 * that cannot pay for the device-wide synchronisation cudaMalloc and cudaFree
 * imply.  The caller passes inputs and outputs already in device memory in
 * the formats below; the function itself calls no cudaMalloc, cudaFree or
 * other allocating routine.
 *
 * The mixed-precision kernels still need scratch (walk descriptors, work
 * order, queue cursor, FP64 re-test records).  It lives in one static device
 * array of about 2.6 MB that every GPU loading the library keeps until the
 * process exits, sized for at most PGF_NOALLOC_MAX_WALKS walks per call;
 * larger calls return PGF_ERR_CAPACITY.  The first call on each device looks
 * up that array's device address (with the device current) and keeps it; make
 * that first call before any stream capture, and do not reset the device
 * (cudaDeviceReset) while the library is in use, since the kept address would
 * then be stale.  All calls share the array: calls on one stream are ordered
 * and safe, calls whose work overlaps on the GPU (other streams, other host
 * threads) race and corrupt each other's results.
 *
 * Every call blocks the calling thread: walk rows and ids are checked on the
 * device first, and the call copies the check's result to the host and waits
 * on the stream for it (so it also waits for the work queued on the stream
 * before it) before it launches the force kernels.  Those are then left
 * running on the stream.  They contain no waits and report no device errors,
 * so the check is the only device-side failure the call can report.
 *
 * walk_table: 6 int64 per walk: i_begin, n_i, epj_begin, n_epj, spj_begin,
 *   n_spj (rows of epi; offsets into id_epj / id_spj).
 * epi: 4 doubles per i-particle: x, y, z, r_search.
 * epj: pgf_epj_device records; epj_r_search: the FP64 r_search of each.
 * spj: pgf_spj_device records.
 * accp: 4 doubles per i-particle: acc x, y, z, pot (G applied); n_ngb: one
 *   int per i-particle.  Rows that no walk covers are left untouched.
 * epi, epj, spj and accp must be 32-byte aligned, walk_table and epj_r_search
 * 8-byte aligned, id_epj, id_spj and n_ngb 4-byte aligned (PGF_ERR_ARG
 * otherwise).  cuda_stream is a cudaStream_t passed as void* that belongs to
 * the current device (PGF_ERR_ARG otherwise); NULL is the legacy default
 * stream.  errbuf (optional, errbuf_len bytes) receives a message on failure. */
#define PGF_NOALLOC_MAX_WALKS 16384

typedef struct pgf_epj_device { /* 32 bytes */
    double pos[3];
    float mass;
    float r_search2;      /* (float)(r_search * r_search), the square taken in double */
} pgf_epj_device;

typedef struct pgf_spj_device { /* 64 bytes */
    double pos[3];
    float mass;
    float pad0;
    float quad_traceless[6]; /* 3q - tr(q) I of the raw second moment q: xx, yy, zz, xy, xz, yz */
    float trace;             /* tr(q) */
    float pad1;
} pgf_spj_device;

int pgf_force_device_noalloc(int n_walk, const int64_t *walk_table, const double *epi, int64_t n_epi_total,
                             const pgf_epj_device *epj, const double *epj_r_search, int64_t n_epj_total,
                             const pgf_spj_device *spj, int64_t n_spj_total, const int *id_epj, int64_t n_id_epj,
                             const int *id_spj, int64_t n_id_spj, double eps2, double rcut2, double G,
                             double *accp, int *n_ngb, void *cuda_stream, char *errbuf, size_t errbuf_len);

/* Releases device and pinned host memory. */
int pgf_finalize(void);

/* ---- Device-resident tree step ---------------------------------------------
 *
 * PeTar's tree step passes every particle through the host: treeSoftForce
 * (src/petar.hpp:879-907) has FDPS build the tree and the interaction lists
 * and hand them to the GPU functor, and kickOne (src/petar.hpp:1198-1212) and
 * driftSingle (src/petar.hpp:1326-1340) update velocities and positions on the
 * host.  A pgf_nbody keeps the particles on the device and runs the whole
 * cycle there, for singles without a hard part:
 *
 *   kick(dt/2), drift(dt), tree + lists, soft force, kick(dt/2)
 *
 * The tree and lists are those of the host list builder that stands in for
 * FDPS (Morton order, n_leaf_limit, n_group_limit, theta opening with the
 * symmetric r_search test), built on the device entry for entry the same.
 * pgf_nbody_run with use_graph != 0 captures its n_steps steps in one CUDA
 * graph (kept for later calls with the same n_steps and dt).
 *
 * These calls report failures through pgf_nbody_last_error().  A handle
 * belongs to the device that was current at creation; calls on one handle
 * must not overlap. */
typedef struct pgf_nbody pgf_nbody;

typedef struct pgf_nbody_config {
    double eps2;              /* softening squared (EPISoft::eps^2) */
    double r_out;             /* changeover outer radius: the cutoff (rcut2 = r_out^2) */
    double G;                 /* gravitational constant */
    double theta;             /* opening angle; <= 0 opens every cell */
    int n_leaf_limit;         /* a cell splits while it holds more particles */
    int n_group_limit;        /* i-groups hold at most this many particles (or are leaves) */
    int precision;            /* PGF_PRECISION_MIXED or PGF_PRECISION_FP64 */
    int kernel_variant;       /* as pgf_set_kernel_variant, TMA variants excluded; -1 = PGF_DEFAULT_KERNEL_VARIANT */
    double list_capacity_factor; /* room kept for growth of cells and lists (>= 1; 0 = 2) */
} pgf_nbody_config;

typedef struct pgf_nbody_stats {
    int64_t n_cells, n_groups;                  /* tree of the last build */
    int64_t n_epj_entries, n_spj_entries;       /* list entries of the last build */
    int64_t interactions_epep, interactions_epsp; /* sum over groups of n_i * n_j, last build */
    int64_t total_epep, total_epsp;             /* the same summed over every build */
    int64_t steps;                              /* steps run so far */
    double last_tree_ms, last_force_ms;         /* split of the last pgf_nbody_force call */
    int kernel_variant;
    int cap_cells;
    int64_t cap_epj_entries, cap_spj_entries;
} pgf_nbody_stats;

/* Copies the particles (pos/vel: 3 doubles each) to the device, builds the
 * tree and lists once (sizing the list arrays from it) and evaluates the
 * forces.  On success *out is the new handle. */
int pgf_nbody_create(const pgf_nbody_config *cfg, int64_t n, const double *pos, const double *vel,
                     const double *mass, const double *r_search, pgf_nbody **out);
/* Tree, lists and forces at the current positions (no kick); waits. */
int pgf_nbody_force(pgf_nbody *h);
/* n_steps kick-drift-force-kick steps of size dt; waits.  *ms (optional)
 * receives the device time of the whole run. */
int pgf_nbody_run(pgf_nbody *h, int n_steps, double dt, int use_graph, double *ms);
/* Copies state back (any pointer may be NULL): pos, vel, acc (3 doubles each),
 * pot (G applied, self pair included as the kernels count it), n_ngb. */
int pgf_nbody_get(pgf_nbody *h, double *pos, double *vel, double *acc, double *pot, int32_t *n_ngb);
/* Replaces positions and/or velocities (NULL keeps them). */
int pgf_nbody_set_state(pgf_nbody *h, const double *pos, const double *vel);
/* Kinetic energy and soft potential energy 1/2 sum m (pot + G m / r_out) of
 * the last forces. */
int pgf_nbody_energy(pgf_nbody *h, double *kinetic, double *potential);
int pgf_nbody_get_stats(pgf_nbody *h, pgf_nbody_stats *stats);
/* The last build's tree and lists in the host builder's form: order[n]
 * (sorted position -> particle index), group_begin, epj_disp and spj_disp
 * [n_groups + 1], id_epj, id_spj, and per cell mass, centre of mass[3],
 * second moment[6] and level.  Any pointer may be NULL. */
int pgf_nbody_export_lists(pgf_nbody *h, int64_t *order, int64_t *group_begin, int64_t *epj_disp,
                           int64_t *spj_disp, int32_t *id_epj, int32_t *id_spj, double *cell_mass,
                           double *cell_pos, double *cell_quad, int32_t *cell_level);
/* Times every available variant on the resident lists and keeps the fastest. */
int pgf_nbody_autotune(pgf_nbody *h, int repeats, int *best_variant, double *best_ms);
/* Changes n_group_limit (the largest i-group) and rebuilds the tree and lists
 * at the current positions, then evaluates the forces.  Larger groups share
 * one interaction list among more i-particles (fewer, longer walks and more
 * interactions per particle), as FDPS's n_group_limit does; PeTar picks it per
 * instruction set (1024 with AVX-512, 512 with AVX2, src/petar.hpp:155-159).
 * The lists, and so the result, depend on it. */
int pgf_nbody_set_group_limit(pgf_nbody *h, int n_group_limit);
/* Autotuner over n_group_limit: for each candidate (NULL / 0 candidates:
 * 256, 512, 1024, 2048) it rebuilds the lists, picks the kernel variant
 * (mixed precision), and times tree + lists + force of one evaluation
 * (`repeats` timed runs); step_ms[c] and interactions[c] (optional, n_limits
 * each) receive the time and the EP-EP + EP-SP interactions per evaluation.
 * Keeps the fastest candidate and its variant, and reports them. */
int pgf_nbody_autotune_groups(pgf_nbody *h, const int *limits, int n_limits, int repeats, double *step_ms,
                              int64_t *interactions, int *best_limit, int *best_variant, double *best_ms);
/* Per-step sample: after every force evaluation (pgf_nbody_force and each
 * step of pgf_nbody_run, graphs included) the n_sample given particles get a
 * record with the mixed-precision result and an FP64 evaluation over the same
 * lists (the plain FP64 kernel's pair formulas), up to max_records
 * evaluations.  n_sample = 0 turns it off.  Changing it drops a captured
 * graph. */
typedef struct pgf_nbody_sample {
    double acc[3], pot;        /* mixed precision, as pgf_nbody_get returns them */
    double acc64[3], pot64;    /* FP64 over the same lists */
    int32_t n_ngb, n_ngb64;
    int32_t record, pad;       /* evaluation index since pgf_nbody_set_sample */
} pgf_nbody_sample;
int pgf_nbody_set_sample(pgf_nbody *h, int n_sample, const int64_t *particles, int max_records);
/* *n_records evaluations recorded so far; out (optional) receives them,
 * record-major: out[r * n_sample + q] (room for max_records * n_sample). */
int pgf_nbody_get_sample(pgf_nbody *h, int *n_records, pgf_nbody_sample *out);
int pgf_nbody_destroy(pgf_nbody *h);
const char *pgf_nbody_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* PETAR_GPUFORCE_H */
