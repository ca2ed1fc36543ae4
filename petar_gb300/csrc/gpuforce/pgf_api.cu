// Host side of the soft-force C ABI (include/petar_gpuforce.h).
//
// Replaces the reference functors' host code (src/force_gpu_cuda.cu:535-880):
// the caller's FDPS records are packed with OpenMP into pinned staging
// buffers in the device layout of pgf_internal.cuh, copied with asynchronous
// cudaMemcpyAsync on one stream, and all walks of a dispatch run in one
// persistent launch.  Dispatch returns once the work is queued; retrieve
// waits, copies the results back and unpacks them into the caller's
// ForceSoft records (overwriting acc, pot and n_ngb as the reference does).
//
// Device buffers are process-wide like the reference's file-static
// cudaPointer objects (src/force_gpu_cuda.cu:513-533), but they grow on demand
// instead of being capped at NI_LIMIT / NJ_LIMIT.
#include "petar_gpuforce.h"
#include "pgf_internal.cuh"

#include <cudaTypedefs.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

namespace {

using namespace pgf;

constexpr int kMaxTags = 16;
constexpr int kMaxChunks = 8;                       // pipeline stages of a large dispatch
constexpr int64_t kChunkIdEntries = 12 << 20;       // about 48 MB of id lists per stage
constexpr int kScratchInts = 8 + 2 * kMaxChunks;
constexpr int kHdErrWords = 4;  // HdWalkArgs::err
static_assert(PGF_NUM_KERNEL_VARIANTS == 1 + kNumWsVariants, "variant 0 plus the warp-specialised variants");
constexpr int64_t kMaxRows = 0x7fffffff;

std::string g_error;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_error = buf;
    return code;
}

#define PGF_CUDA(call)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return fail(PGF_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));         \
    } while (0)

template <class T>
struct DevBuf {
    T* d = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap && d) return cudaSuccess;
        size_t want = std::max<size_t>(n, cap + cap / 2);
        if (want == 0) want = 1;
        if (d) cudaFree(d);
        d = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&d, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (d) cudaFree(d);
        d = nullptr;
        cap = 0;
    }
};

template <class T>
struct HostBuf {
    T* h = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t n) {
        if (n <= cap && h) return cudaSuccess;
        size_t want = std::max<size_t>(n, cap + cap / 2);
        if (want == 0) want = 1;
        if (h) cudaFreeHost(h);
        h = nullptr;
        cap = 0;
        cudaError_t e = cudaMallocHost(&h, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (h) cudaFreeHost(h);
        h = nullptr;
        cap = 0;
    }
};

struct TagState {
    bool dispatched = false;  // dispatched and not yet retrieved
    bool has_data = false;    // device holds a complete dispatch (for recompute)
    int n_walk = 0;
    int64_t ni_tot = 0;
    int precision = PGF_PRECISION_MIXED;
    int variant = 0;
    int mode = PGF_MODE_FORCE;
    std::vector<int> n_epi;
    std::vector<int64_t> epi_disp;
    DevBuf<EpiDev> epi;
    DevBuf<int32_t> id_epj, id_spj, order;
    DevBuf<WalkDesc> walks;
    DevBuf<Accp> accp;
    DevBuf<int32_t> nnb;
    HostBuf<EpiDev> h_epi;
    HostBuf<int32_t> h_id_epj, h_id_spj, h_order;
    HostBuf<WalkDesc> h_walks;
    HostBuf<Accp> h_accp;
    HostBuf<int32_t> h_nnb;
    HostBuf<int32_t> h_flags;  // queue head, n_retest, err, re-tested records
    DevBuf<CoRec> epi_co;      // fused changeover mode
    HostBuf<CoRec> h_epi_co;
    DevBuf<double> pot_soft;
    HostBuf<double> h_pot_soft;
    DevBuf<Accp> epi_acc;  // gradient mode: EPI accelerations in, acorr out
    HostBuf<Accp> h_epi_acc;
    DevBuf<Accp> acorr;
    HostBuf<Accp> h_acorr;
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    // Pipelined dispatch, per stage: copy start/end, main kernel start/end,
    // stage done (after the re-test kernel), results copied back.
    cudaEvent_t evc[kMaxChunks][6] = {};
    int n_chunks = 0;  // stages of the last dispatch (0: a single launch)
    std::vector<int32_t> ord;  // layout position -> walk
    std::vector<int> stage_k;  // stage boundaries in layout positions
    std::vector<int64_t> stage_i;  // and in EPI rows
    bool times_pending = false;  // kernel events recorded, not yet added to the profile
    Params params{};
    // Walks split over several CTAs (single-launch dispatches only).
    int n_split = 0;
    DevBuf<SplitRec> splits;
    HostBuf<SplitRec> h_splits;
    // Host-direct tables, read by the kernels in place: where the gather
    // kernel reads each walk, and where the scatter kernel writes its
    // results; h_hd_err receives the gather's id-check outcome.
    HostBuf<WalkSrc> h_src;
    HostBuf<ForceDst> h_dst;
    HostBuf<int32_t> h_hd_err;
    cudaEvent_t ev_in = nullptr;  // host-direct dispatch: the gather has read the caller's arrays
};

struct State {
    bool init = false;
    int device = -1;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // host-to-device copies of pipelined dispatches
    cudaStream_t stage_stream[kMaxChunks] = {};  // kernels of pipeline stages
    cudaStream_t d2h_stream = nullptr;             // results of pipeline stages back
    bool user_stream = false;
    double eps2 = 0, rcut2 = 0, G = 1;
    int precision = PGF_PRECISION_MIXED;
    int variant = PGF_DEFAULT_KERNEL_VARIANT;  // mixed-precision kernel variant (pgf_set_kernel_variant)
    int stages = 0;   // dispatch pipeline stages (pgf_set_dispatch_stages); 0 = by size
    bool walk_split = true;  // split the largest walks of small dispatches (pgf_set_walk_split)
    int split_div = 16;      // split unit: 1/split_div of one SM's even share (pgf_autotune_dispatch)
    int gr_compensated = 1;  // gradient pass far pairs: 1 compensated r^2 and 1/r (default), 0 FP32
    uint64_t wait_limit_ns = 0;  // bounded waits of the kernels (pgf_set_wait_limit_ns; 0: 1 s)
    int stall_after_items = 0;   // test hook (pgf_test_stall_producer)
    // Host-direct data movement (pgf_set_host_direct): the device reads the
    // caller's records in place and writes results into them; used when the
    // device can access pageable host memory.
    bool hd_supported = false;
    bool hd_enabled = true;
    int mode = PGF_MODE_FORCE;
    // shared j data
    DevBuf<EpjMix> epj;
    DevBuf<double> epj_m64, epj_rs64;
    DevBuf<SpjMix> spj;
    DevBuf<SpjQ64> spj_q64;
    DevBuf<EpjF32> epj32;  // (hi, lo) FP32 copies built on the device
    DevBuf<SpjF32> spj32;
    TensorMaps tmaps;      // TMA descriptors of epj32 / spj32
    bool co_set = false;   // changeover layout given (pgf_set_changeover_layout)
    pgf_changeover_layout co{};
    bool j_co_sent = false;  // the last send packed the EPJ changeover records
    DevBuf<CoRec> epj_co;
    HostBuf<CoRec> h_epj_co;
    bool gr_set = false;  // gradient layout given (pgf_set_gradient_layout)
    pgf_gradient_layout gr{};
    bool j_gr_sent = false;
    DevBuf<AccF32> epj_acc32;
    HostBuf<AccF32> h_epj_acc32;
    HostBuf<EpjMix> h_epj;
    HostBuf<double> h_epj_m64, h_epj_rs64;
    HostBuf<SpjMix> h_spj;
    HostBuf<SpjQ64> h_spj_q64;
    int64_t n_epj_tot = 0, n_spj_tot = 0;
    bool j_sent = false;
    // scratch
    // [0] queue head, [1] n_retest (single launch), [2] err, [3] re-tested
    // records, [8 + 2s], [9 + 2s]: queue head and n_retest of pipeline stage s
    DevBuf<int32_t> scratch;
    DevBuf<Retest> retest;
    int retest_cap = 0;
    DevBuf<int32_t> hd_err;  // per tag: id check of its last host-direct dispatch (HdWalkArgs::err)
    std::vector<double> walk_rcut2;
    TagState tags[kMaxTags];
    pgf_profile prof{};
    cudaEvent_t ev_send0 = nullptr, ev_send1 = nullptr;
    bool send_pending = false;  // j copies queued, time not yet in the profile
};

State g;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int ensure_init() {
    if (!g.init) return fail(PGF_ERR_STATE, "pgf_initialize has not been called");
    return PGF_OK;
}

// Whether this call moves data host-direct (supported and not turned off).
bool use_hd() { return g.hd_supported && g.hd_enabled; }

// The host-direct kernels load and store the records' FP64 and integer
// fields in place, so they take only naturally aligned records: 8-byte
// aligned arrays whose record size and field offsets are multiples of 8 (and
// at most 4 KB per EPI record, the gather's staging).  Anything else takes
// the host packing path.
inline bool al8(size_t v) { return (v & 7) == 0; }
inline bool al8p(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 7) == 0; }

bool hd_send_ok(const void* epj, int64_t n_epj, const pgf_epj_layout* el, const void* spj, int64_t n_spj,
                const pgf_spj_layout* sl) {
    if (n_epj > 0) {
        if (!al8p(epj) || !al8(el->size) || !al8(el->off_mass) || !al8(el->off_pos) || !al8(el->off_r_search))
            return false;
        if (g.co_set && !(al8(g.co.epj_off_id) && al8(g.co.epj_off_r_in) && al8(g.co.epj_off_r_out) &&
                          al8(g.co.epj_off_mass_backup) && al8(g.co.epj_off_status)))
            return false;
        if (g.gr_set && !al8(g.gr.epj_off_acc)) return false;
    }
    if (n_spj > 0 && (!al8p(spj) || !al8(sl->size) || !al8(sl->off_mass) || !al8(sl->off_pos) ||
                      (sl->has_quad && !al8(sl->off_quad))))
        return false;
    return true;
}

bool hd_walks_ok(int n_walk, const void* const* epi, const int* n_epi, const pgf_epi_layout* il,
                 const int* const* id_epj, const int* n_epj, const int* const* id_spj, const int* n_spj, int mode) {
    if (n_walk <= 0) return true;
    if (!al8(il->size) || il->size > 4096 || !al8(il->off_pos) || !al8(il->off_r_search)) return false;
    if (mode == PGF_MODE_GRADIENT && !al8(g.gr.epi_off_acc)) return false;
    if (mode == PGF_MODE_FORCE_CHANGEOVER && !(al8(g.co.epi_off_id) && al8(g.co.epi_off_r_in) &&
                                               al8(g.co.epi_off_r_out) && al8(g.co.epi_off_self_mass)))
        return false;
    for (int w = 0; w < n_walk; ++w) {
        if (n_epi[w] > 0 && !al8p(epi[w])) return false;
        if (n_epj[w] > 0 && (reinterpret_cast<uintptr_t>(id_epj[w]) & 3)) return false;
        if (n_spj[w] > 0 && (reinterpret_cast<uintptr_t>(id_spj[w]) & 3)) return false;
    }
    return true;
}

bool hd_force_ok(int n_walk, const int* ni, void* const* force, const pgf_force_layout* fl, int mode) {
    if (n_walk <= 0) return true;
    if (!al8(fl->size) || !al8(fl->off_acc) || !al8(fl->off_pot) || fl->off_n_ngb % (size_t)fl->n_ngb_bytes)
        return false;
    if (mode == PGF_MODE_GRADIENT && !al8(g.gr.force_off_acorr)) return false;
    if (mode == PGF_MODE_FORCE_CHANGEOVER && !al8(g.co.force_off_pot_soft)) return false;
    for (int w = 0; w < n_walk; ++w)
        if (ni[w] > 0 && !al8p(force[w])) return false;
    return true;
}

int setup_device(int rank) {
    int ngpu = 0;
    cudaError_t e = cudaGetDeviceCount(&ngpu);
    if (e != cudaSuccess || ngpu <= 0) {
        cudaGetLastError();
        return fail(PGF_ERR_NO_DEVICE, "no CUDA device available (%s)",
                    e == cudaSuccess ? "device count 0" : cudaGetErrorString(e));
    }
    g.device = (rank < 0 ? -rank : rank) % ngpu;
    PGF_CUDA(cudaSetDevice(g.device));
    PGF_CUDA(cudaDeviceGetAttribute(&g.num_sms, cudaDevAttrMultiProcessorCount, g.device));
    int pageable = 0;
    PGF_CUDA(cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, g.device));
    g.hd_supported = pageable != 0;
    PGF_CUDA(cudaStreamCreateWithFlags(&g.own_stream, cudaStreamNonBlocking));
    PGF_CUDA(cudaStreamCreateWithFlags(&g.copy_stream, cudaStreamNonBlocking));
    for (auto& st : g.stage_stream) PGF_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    PGF_CUDA(cudaStreamCreateWithFlags(&g.d2h_stream, cudaStreamNonBlocking));
    if (!g.user_stream) g.stream = g.own_stream;
    PGF_CUDA(cudaEventCreate(&g.ev_send0));
    PGF_CUDA(cudaEventCreate(&g.ev_send1));
    for (auto& t : g.tags) {
        PGF_CUDA(cudaEventCreate(&t.ev_in));
        for (auto& ev : t.ev) PGF_CUDA(cudaEventCreate(&ev));
        for (auto& c : t.evc)
            for (auto& ev : c) PGF_CUDA(cudaEventCreate(&ev));
    }
    PGF_CUDA(g.scratch.ensure(kScratchInts));
    g.retest_cap = 1 << 20;
    PGF_CUDA(g.retest.ensure((size_t)g.retest_cap));
    PGF_CUDA(cudaMemset(g.scratch.d, 0, kScratchInts * sizeof(int32_t)));
    PGF_CUDA(g.hd_err.ensure(kHdErrWords * kMaxTags));
    PGF_CUDA(cudaMemset(g.hd_err.d, 0, kHdErrWords * kMaxTags * sizeof(int32_t)));
    g.init = true;
    return PGF_OK;
}

// Smallest float not below v (v >= 0).
inline float round_up(double v) {
    float f = (float)v;
    if ((double)f < v) f = std::nextafter(f, HUGE_VALF);
    return f;
}

inline const double* dptr(const void* base, size_t off) {
    return reinterpret_cast<const double*>(reinterpret_cast<const char*>(base) + off);
}

inline int64_t i64at(const char* r, size_t off) {
    int64_t v;
    std::memcpy(&v, r + off, sizeof(v));
    return v;
}

// Changeover record of one particle: the derived ChangeOver members of
// src/changeover.hpp:64-75 in FP64, rounded to FP32.
inline CoRec make_co(double r_in, double r_out, double mass, int64_t id) {
    CoRec c;
    const double norm = 1.0 / (r_out - r_in);
    const double coff = (r_out - r_in) / (r_out + r_in);
    c.r_in = (float)r_in;
    c.r_out = (float)r_out;
    c.norm = (float)norm;
    c.coff = (float)coff;
    c.pot_off = (float)((1.0 + coff) / r_out);
    c.mass = (float)mass;
    c.id = id;
    return c;
}

// 2-D tensor map over n rows of `row_floats` floats, boxes one row high (the
// form TMA gather4 loads take).
int encode_rows(CUtensorMap* map, void* base, int64_t n, int row_floats) {
    const cuuint64_t dims[2] = {(cuuint64_t)row_floats, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)row_floats * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)row_floats, 1};
    const cuuint32_t estr[2] = {1, 1};
    // The driver entry point is looked up through the runtime, so the library
    // does not link libcuda and loads on hosts without a driver.
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q{};
        void* fn = nullptr;
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return fail(PGF_ERR_CUDA, "cuTensorMapEncodeTiled not available from the driver");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, base, dims, strides, box, estr,
                              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
                              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(PGF_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return PGF_OK;
}

// Rebuilds the TMA descriptors of the (hi, lo) j arrays after a send.
int encode_tensor_maps(int64_t n_epj, int64_t n_spj) {
    g.tmaps.valid = false;
    std::memset(&g.tmaps.epj, 0, sizeof(CUtensorMap));
    std::memset(&g.tmaps.spj, 0, sizeof(CUtensorMap));
    if (n_epj > 0)
        if (int r = encode_rows(&g.tmaps.epj, g.epj32.d, n_epj, (int)(sizeof(EpjF32) / sizeof(float)))) return r;
    if (n_spj > 0)
        if (int r = encode_rows(&g.tmaps.spj, g.spj32.d, n_spj, (int)(sizeof(SpjF32) / sizeof(float)))) return r;
    g.tmaps.valid = true;
    return PGF_OK;
}

// Adds the time of the last j send to the profile once its copies are done.
void harvest_send(bool wait = false) {
    if (!g.send_pending) return;
    if (wait) cudaEventSynchronize(g.ev_send1);
    if (cudaEventQuery(g.ev_send1) != cudaSuccess) return;
    float ms = 0;
    cudaEventElapsedTime(&ms, g.ev_send0, g.ev_send1);
    g.prof.send += 1e-3 * ms;
    g.send_pending = false;
}

// The send phase host-direct: one kernel reads the caller's EPJ / SPJ records
// in place and writes every device form of them (the host packing's
// arithmetic), then the call waits for it, since the caller's arrays are only
// valid during the call.
int send_j_host_direct(const void* epj, int64_t n_epj, const pgf_epj_layout* el, const void* spj, int64_t n_spj,
                       const pgf_spj_layout* sl) {
    PGF_CUDA(g.epj.ensure(n_epj));
    PGF_CUDA(g.epj_m64.ensure(n_epj));
    PGF_CUDA(g.epj_rs64.ensure(n_epj));
    PGF_CUDA(g.spj.ensure(n_spj));
    PGF_CUDA(g.spj_q64.ensure(n_spj));
    PGF_CUDA(g.epj32.ensure(n_epj));
    PGF_CUDA(g.spj32.ensure(n_spj));
    const bool co = g.co_set && n_epj > 0, gr = g.gr_set && n_epj > 0;
    if (co) PGF_CUDA(g.epj_co.ensure(n_epj));
    if (gr) PGF_CUDA(g.epj_acc32.ensure(n_epj));
    HdSendArgs a{};
    a.epj = static_cast<const char*>(epj);
    a.n_epj = n_epj;
    if (n_epj > 0) {
        a.epj_size = el->size;
        a.epj_off_mass = el->off_mass;
        a.epj_off_pos = el->off_pos;
        a.epj_off_rs = el->off_r_search;
    }
    a.spj = static_cast<const char*>(spj);
    a.n_spj = n_spj;
    if (n_spj > 0) {
        a.spj_size = sl->size;
        a.spj_off_mass = sl->off_mass;
        a.spj_off_pos = sl->off_pos;
        a.spj_off_quad = sl->off_quad;
        a.spj_has_quad = sl->has_quad;
    }
    if (co) {
        a.co_epj_off_id = g.co.epj_off_id;
        a.co_epj_off_r_in = g.co.epj_off_r_in;
        a.co_epj_off_r_out = g.co.epj_off_r_out;
        a.co_epj_off_mass_backup = g.co.epj_off_mass_backup;
        a.co_epj_off_status = g.co.epj_off_status;
        a.out_epj_co = g.epj_co.d;
    }
    if (gr) {
        a.gr_epj_off_acc = g.gr.epj_off_acc;
        a.out_epj_acc32 = g.epj_acc32.d;
    }
    a.out_epj = g.epj.d;
    a.out_epj_m64 = g.epj_m64.d;
    a.out_epj_rs64 = g.epj_rs64.d;
    a.out_epj32 = g.epj32.d;
    a.out_spj = g.spj.d;
    a.out_spj_q64 = g.spj_q64.d;
    a.out_spj32 = g.spj32.d;
    PGF_CUDA(cudaEventRecord(g.ev_send0, g.stream));
    {
        const cudaError_t e = launch_gather_j(a, g.num_sms, g.stream);
        if (e != cudaSuccess) return fail(PGF_ERR_CUDA, "j gather kernel failed: %s", cudaGetErrorString(e));
    }
    PGF_CUDA(cudaEventRecord(g.ev_send1, g.stream));
    g.j_co_sent = co;
    g.j_gr_sent = gr;
    if (int r = encode_tensor_maps(n_epj, n_spj)) return r;
    PGF_CUDA(cudaEventSynchronize(g.ev_send1));
    g.send_pending = true;
    harvest_send();
    g.n_epj_tot = n_epj;
    g.n_spj_tot = n_spj;
    g.j_sent = true;
    return PGF_OK;
}

// Packs the shared EPJ / SPJ arrays (the send_flag phase,
// src/force_gpu_cuda.cu:577-619).
int pack_and_send_j(const void* epj, int64_t n_epj, const pgf_epj_layout* el, const void* spj,
                    int64_t n_spj, const pgf_spj_layout* sl) {
    if (n_epj < 0 || n_spj < 0) return fail(PGF_ERR_ARG, "negative EPJ/SPJ count");
    if ((n_epj > 0 && (!epj || !el)) || (n_spj > 0 && (!spj || !sl)))
        return fail(PGF_ERR_ARG, "EPJ/SPJ array or layout is NULL");
    // Kernels of earlier dispatches may still read the device j arrays and
    // pending copies may still read the pinned staging: finish them before
    // either is reused or reallocated.
    PGF_CUDA(cudaStreamSynchronize(g.stream));
    harvest_send();
    if (use_hd() && hd_send_ok(epj, n_epj, el, spj, n_spj, sl))
        return send_j_host_direct(epj, n_epj, el, spj, n_spj, sl);
    const double t0 = now_s();
    PGF_CUDA(g.h_epj.ensure(n_epj));
    PGF_CUDA(g.h_epj_m64.ensure(n_epj));
    PGF_CUDA(g.h_epj_rs64.ensure(n_epj));
    PGF_CUDA(g.h_spj.ensure(n_spj));
    PGF_CUDA(g.h_spj_q64.ensure(n_spj));
    PGF_CUDA(g.epj.ensure(n_epj));
    PGF_CUDA(g.epj_m64.ensure(n_epj));
    PGF_CUDA(g.epj_rs64.ensure(n_epj));
    PGF_CUDA(g.spj.ensure(n_spj));
    PGF_CUDA(g.spj_q64.ensure(n_spj));
    PGF_CUDA(g.epj32.ensure(n_epj));
    PGF_CUDA(g.spj32.ensure(n_spj));
    g.j_co_sent = false;
    g.j_gr_sent = false;
    if (g.gr_set && n_epj > 0) {
        PGF_CUDA(g.h_epj_acc32.ensure(n_epj));
        PGF_CUDA(g.epj_acc32.ensure(n_epj));
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < n_epj; ++j) {
            const char* r = reinterpret_cast<const char*>(epj) + j * el->size;
            const double* a = dptr(r, g.gr.epj_off_acc);
            AccF32 o;
            o.xh = (float)a[0];
            o.yh = (float)a[1];
            o.zh = (float)a[2];
            o.xl = (float)(a[0] - (double)o.xh);
            o.yl = (float)(a[1] - (double)o.yh);
            o.zl = (float)(a[2] - (double)o.zh);
            o.pad0 = o.pad1 = 0.f;
            g.h_epj_acc32.h[j] = o;
        }
    }
    if (g.co_set && n_epj > 0) {
        PGF_CUDA(g.h_epj_co.ensure(n_epj));
        PGF_CUDA(g.epj_co.ensure(n_epj));
        const pgf_changeover_layout& L = g.co;
#pragma omp parallel for schedule(static)
        for (int64_t j = 0; j < n_epj; ++j) {
            const char* r = reinterpret_cast<const char*>(epj) + j * el->size;
            const double status = *dptr(r, L.epj_off_status), mbk = *dptr(r, L.epj_off_mass_backup);
            // Mass of the pair potential of a neighbour (src/hard.hpp:1458-1476):
            // singles their mass, members their backup mass, others none.
            const double m_pot = (status == 0.0 && mbk == 0.0) ? *dptr(r, el->off_mass) : (status < 0.0 ? mbk : 0.0);
            g.h_epj_co.h[j] = make_co(*dptr(r, L.epj_off_r_in), *dptr(r, L.epj_off_r_out), m_pot, i64at(r, L.epj_off_id));
        }
    }
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n_epj; ++j) {
        const char* r = reinterpret_cast<const char*>(epj) + j * el->size;
        const double* p = dptr(r, el->off_pos);
        const double rs = *dptr(r, el->off_r_search);
        const double m = *dptr(r, el->off_mass);
        g.h_epj.h[j] = EpjMix{p[0], p[1], p[2], (float)m, (float)(rs * rs)};
        g.h_epj_m64.h[j] = m;
        g.h_epj_rs64.h[j] = rs;
    }
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < n_spj; ++j) {
        const char* r = reinterpret_cast<const char*>(spj) + j * sl->size;
        const double* p = dptr(r, sl->off_pos);
        const double m = *dptr(r, sl->off_mass);
        double q[6] = {0, 0, 0, 0, 0, 0};
        if (sl->has_quad) {
            const double* qq = dptr(r, sl->off_quad);
            for (int k = 0; k < 6; ++k) q[k] = qq[k];
        }
        // Traceless form in FP64, then rounded once (see pgf_kernels_mixed.cu).
        const double tr = q[0] + q[1] + q[2];
        SpjMix s;
        s.x = p[0];
        s.y = p[1];
        s.z = p[2];
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
        g.h_spj.h[j] = s;
        SpjQ64 d;
        d.m = m;
        for (int k = 0; k < 6; ++k) d.q[k] = q[k];
        d.pad = 0.0;
        g.h_spj_q64.h[j] = d;
    }
    g.prof.copy += now_s() - t0;
    PGF_CUDA(cudaEventRecord(g.ev_send0, g.stream));
    if (n_epj) {
        PGF_CUDA(cudaMemcpyAsync(g.epj.d, g.h_epj.h, n_epj * sizeof(EpjMix), cudaMemcpyHostToDevice, g.stream));
        PGF_CUDA(cudaMemcpyAsync(g.epj_m64.d, g.h_epj_m64.h, n_epj * sizeof(double), cudaMemcpyHostToDevice,
                                 g.stream));
        PGF_CUDA(cudaMemcpyAsync(g.epj_rs64.d, g.h_epj_rs64.h, n_epj * sizeof(double), cudaMemcpyHostToDevice,
                                 g.stream));
    }
    if (n_spj) {
        PGF_CUDA(cudaMemcpyAsync(g.spj.d, g.h_spj.h, n_spj * sizeof(SpjMix), cudaMemcpyHostToDevice, g.stream));
        PGF_CUDA(cudaMemcpyAsync(g.spj_q64.d, g.h_spj_q64.h, n_spj * sizeof(SpjQ64), cudaMemcpyHostToDevice,
                                 g.stream));
    }
    if (g.co_set && n_epj > 0) {
        PGF_CUDA(cudaMemcpyAsync(g.epj_co.d, g.h_epj_co.h, n_epj * sizeof(CoRec), cudaMemcpyHostToDevice, g.stream));
        g.j_co_sent = true;
    }
    if (g.gr_set && n_epj > 0) {
        PGF_CUDA(cudaMemcpyAsync(g.epj_acc32.d, g.h_epj_acc32.h, n_epj * sizeof(AccF32), cudaMemcpyHostToDevice,
                                 g.stream));
        g.j_gr_sent = true;
    }
    {
        const cudaError_t e = launch_split_j(g.epj.d, n_epj, g.epj32.d, g.spj.d, n_spj, g.spj32.d, g.stream);
        if (e != cudaSuccess) return fail(PGF_ERR_CUDA, "j split kernel failed: %s", cudaGetErrorString(e));
    }
    if (int r = encode_tensor_maps(n_epj, n_spj)) return r;
    // The copies run behind the caller's next steps (walk packing); the
    // staging is not written again before the next send, which waits first.
    PGF_CUDA(cudaEventRecord(g.ev_send1, g.stream));
    g.send_pending = true;
    g.n_epj_tot = n_epj;
    g.n_spj_tot = n_spj;
    g.j_sent = true;
    return PGF_OK;
}

// Scratch of a single launch (stage < 0) or of pipeline stage `stage` of
// n_stages: its own queue cursor, re-test counter and slice of the re-test
// records, so that the launches of different stages may overlap.
void bind_scratch(Params& p, int stage = -1, int n_stages = 1) {
    p.wait_limit_ns = g.wait_limit_ns;
    p.stall_after_items = g.stall_after_items;
    p.err = g.scratch.d + 2;
    p.retest_total = g.scratch.d + 3;
    if (stage < 0) {
        p.queue_head = g.scratch.d;
        p.n_retest = g.scratch.d + 1;
        p.retest = g.retest.d;
        p.retest_cap = g.retest_cap;
    } else {
        const int cap = g.retest_cap / n_stages;
        p.queue_head = g.scratch.d + 8 + 2 * stage;
        p.n_retest = g.scratch.d + 9 + 2 * stage;
        p.retest = g.retest.d + (size_t)stage * cap;
        p.retest_cap = cap;
    }
}

// Main kernel of the tag's precision and variant on stream s, bracketed by two
// events, then the FP64 neighbour re-test.
int launch_kernels(const TagState& t, const Params& p, cudaStream_t s, cudaEvent_t ev_start, cudaEvent_t ev_end) {
    PGF_CUDA(cudaEventRecord(ev_start, s));
    cudaError_t e;
    if (t.mode == PGF_MODE_GRADIENT) {
        e = launch_gradient(p, s, g.num_sms);
        if (e == cudaSuccess) e = cudaEventRecord(ev_end, s);
    } else if (t.mode == PGF_MODE_FORCE_CHANGEOVER) {
        e = launch_ws_changeover(p, s, g.num_sms);
        if (e == cudaSuccess) e = cudaEventRecord(ev_end, s);
        if (e == cudaSuccess && p.n_walk > 0) e = launch_retest(p, s, g.num_sms);
    } else if (t.mode == PGF_MODE_NEIGHBOR_SEARCH) {
        e = launch_ws_search(p, s, g.num_sms);
        if (e == cudaSuccess) e = cudaEventRecord(ev_end, s);
        if (e == cudaSuccess && p.n_walk > 0) e = launch_retest(p, s, g.num_sms);
    } else if (t.precision == PGF_PRECISION_FP64) {
        e = launch_fp64(p, s, g.num_sms);
        if (e == cudaSuccess) e = cudaEventRecord(ev_end, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(p.n_retest, 0, sizeof(int32_t), s);
    } else {
        e = t.variant == 0 ? launch_mixed(p, s, g.num_sms) : launch_ws(p, s, g.num_sms, t.variant - 1, &g.tmaps);
        if (e == cudaSuccess) e = cudaEventRecord(ev_end, s);
        if (e == cudaSuccess && p.n_walk > 0) e = launch_retest(p, s, g.num_sms);
    }
    if (e != cudaSuccess) return fail(PGF_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    return PGF_OK;
}

// One launch over all walks of the tag (recompute, small dispatches).
int launch_tag(TagState& t) {
    bind_scratch(t.params);
    if (int r = launch_kernels(t, t.params, g.stream, t.ev[1], t.ev[2])) return r;
    if (t.n_split > 0) {
        const cudaError_t e = launch_combine_parts(t.splits.d, t.n_split, t.params.out_accp, t.params.out_nnb,
                                                   t.params.out_pot_soft, t.params.out_acorr, g.stream);
        if (e != cudaSuccess) return fail(PGF_ERR_CUDA, "combine kernel failed: %s", cudaGetErrorString(e));
    }
    PGF_CUDA(cudaEventRecord(t.ev[3], g.stream));
    t.n_chunks = 0;
    t.dispatched = true;
    t.has_data = true;
    t.times_pending = true;
    return PGF_OK;
}

// Adds the kernel times of the tag's last launch to the profile (once).
void harvest_times(TagState& t) {
    if (!t.times_pending) return;
    float ms_send = 0, ms_calc = 0, ms_main = 0;
    if (t.n_chunks > 0) {
        // Stages overlap: the main-kernel time is the span from the first
        // stage's start to the last main-kernel end.
        cudaEventElapsedTime(&ms_calc, t.evc[0][2], t.ev[3]);
        for (int c = 0; c < t.n_chunks; ++c) {
            float a = 0, b = 0;
            cudaEventElapsedTime(&a, t.evc[c][0], t.evc[c][1]);
            cudaEventElapsedTime(&b, t.evc[0][2], t.evc[c][3]);
            ms_send += a;
            ms_main = std::max(ms_main, b);
        }
    } else {
        cudaEventElapsedTime(&ms_calc, t.ev[1], t.ev[3]);
        cudaEventElapsedTime(&ms_send, t.ev[0], t.ev[1]);
        cudaEventElapsedTime(&ms_main, t.ev[1], t.ev[2]);
    }
    g.prof.send += 1e-3 * ms_send;
    g.prof.calc += 1e-3 * ms_calc;
    g.prof.calc_main += 1e-3 * ms_main;
    g.prof.last_calc = 1e-3 * ms_calc;
    g.prof.last_calc_main = 1e-3 * ms_main;
    t.times_pending = false;
}

// Offsets of one walk in the packed (cost-sorted) layout.
struct Slot3 {
    int64_t i, e, s;
};

// Packs walk w of an index dispatch into position k of the tag's pinned
// staging: its EPI rows, its id lists (validated against the sent arrays in
// the same pass) and its descriptor.  Returns false if an id is out of range.
bool pack_walk(TagState& t, int k, int w, const Slot3& o, const void* const* epi, const int* n_epi,
               const pgf_epi_layout* il, const int* const* id_epj, const int* n_epj, const int* const* id_spj,
               const int* n_spj) {
    double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL};
    double rs_max = 0.0;
    const char* base = reinterpret_cast<const char*>(epi[w]);
    for (int i = 0; i < n_epi[w]; ++i) {
        const char* r = base + (size_t)i * il->size;
        const double* p = dptr(r, il->off_pos);
        EpiDev e{p[0], p[1], p[2], *dptr(r, il->off_r_search)};
        t.h_epi.h[o.i + i] = e;
        if (t.mode == PGF_MODE_GRADIENT) {
            const double* a = dptr(r, g.gr.epi_off_acc);
            t.h_epi_acc.h[o.i + i] = Accp{a[0], a[1], a[2], 0.0};
        }
        if (t.mode == PGF_MODE_FORCE_CHANGEOVER) {
            const pgf_changeover_layout& L = g.co;
            t.h_epi_co.h[o.i + i] = make_co(*dptr(r, L.epi_off_r_in), *dptr(r, L.epi_off_r_out),
                                            *dptr(r, L.epi_off_self_mass), i64at(r, L.epi_off_id));
        }
        rs_max = std::max(rs_max, e.rs);
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], p[d]);
            hi[d] = std::max(hi[d], p[d]);
        }
    }
    unsigned bad = 0;
    {
        const int32_t* src = n_epj[w] ? id_epj[w] : nullptr;
        int32_t* dst = t.h_id_epj.h + o.e;
        const unsigned lim = (unsigned)g.n_epj_tot;
        for (int q = 0; q < n_epj[w]; ++q) {
            const int32_t v = src[q];
            bad |= (unsigned)v >= lim;
            dst[q] = v;
        }
    }
    {
        const int32_t* src = n_spj[w] ? id_spj[w] : nullptr;
        int32_t* dst = t.h_id_spj.h + o.s;
        const unsigned lim = (unsigned)g.n_spj_tot;
        for (int q = 0; q < n_spj[w]; ++q) {
            const int32_t v = src[q];
            bad |= (unsigned)v >= lim;
            dst[q] = v;
        }
    }
    WalkDesc d;
    d.epj_begin = o.e;
    d.spj_begin = o.s;
    d.i_begin = (int32_t)o.i;
    d.n_i = n_epi[w];
    d.n_epj = n_epj[w];
    d.n_spj = n_spj[w];
    if (n_epi[w] > 0) {
        d.cx = 0.5 * (lo[0] + hi[0]);
        d.cy = 0.5 * (lo[1] + hi[1]);
        d.cz = 0.5 * (lo[2] + hi[2]);
        // Half-extents about the centre and the largest r_search, rounded up
        // so the kernel's far-field classification stays conservative.
        d.hx = round_up(std::max(hi[0] - d.cx, d.cx - lo[0]));
        d.hy = round_up(std::max(hi[1] - d.cy, d.cy - lo[1]));
        d.hz = round_up(std::max(hi[2] - d.cz, d.cz - lo[2]));
        d.rs_max = round_up(rs_max);
    } else {
        d.cx = d.cy = d.cz = 0.0;
        d.hx = d.hy = d.hz = d.rs_max = 0.f;
    }
    d.part = 0;
    d.pad[0] = d.pad[1] = d.pad[2] = 0.f;
    d.rcut2 = g.walk_rcut2.empty() ? g.rcut2 : g.walk_rcut2[w];
    t.h_walks.h[k] = d;
    t.h_order.h[k] = k;
    return bad == 0;
}

// A walk of a single-launch dispatch that runs as several parts.
struct SplitPlan {
    int k, parts;
    int64_t rows1;  // first EPI row of part 1
    int desc1;      // layout position of part 1's descriptor
};

// Cost of list slice j of `parts` of a walk (the work-queue order of walks
// and parts): n_i (n_epj + 2 n_spj) of the slice.
inline double part_cost(int n_i, int n_epj, int n_spj, int j, int parts) {
    const int e = (int)((int64_t)n_epj * (j + 1) / parts) - (int)((int64_t)n_epj * j / parts);
    const int s = (int)((int64_t)n_spj * (j + 1) / parts) - (int)((int64_t)n_spj * j / parts);
    return (double)n_i * ((double)e + 2.0 * (double)s);
}

// Work-queue order of a dispatch's walks and parts, most expensive first, in
// linear time: costs are bucketed in eighths of an octave below the largest
// (the 3 leading mantissa bits and the exponent of the double), and equal
// buckets keep their layout order.  The order only decides which CTA runs
// which descriptor, never a result.
void queue_order(const std::vector<std::pair<double, int>>& cq, int32_t* out) {
    constexpr int kBuckets = 256;
    auto key = [](double c) -> int64_t {
        if (!(c > 0.0)) return 0;
        int64_t bits;
        std::memcpy(&bits, &c, sizeof(bits));
        return bits >> 49;  // exponent and 3 mantissa bits: monotonic in c > 0
    };
    const size_t n = cq.size();
    std::vector<int64_t> keys(n);
    int64_t kmax = 0;
    for (size_t k = 0; k < n; ++k) {
        keys[k] = key(cq[k].first);
        kmax = std::max(kmax, keys[k]);
    }
    int count[kBuckets + 1] = {};
    auto bucket = [&](size_t k) { return (int)std::min<int64_t>(kBuckets - 1, kmax - keys[k]); };
    for (size_t k = 0; k < n; ++k) ++count[bucket(k) + 1];
    for (int b = 0; b < kBuckets; ++b) count[b + 1] += count[b];
    for (size_t k = 0; k < n; ++k) out[count[bucket(k)]++] = cq[k].second;
}

// The walk phase of a single-launch index dispatch, host-direct: the host
// writes one table entry per walk (where its EPI records and id lists lie,
// where they go, how it splits), and a gather kernel reads the caller's
// arrays in place, builds the EPI rows, the walk descriptors and the id
// lists, and checks every id against the sent arrays.  The call waits for
// the gather (the caller's arrays are only valid during the call) and reports
// an out-of-range id before any force kernel is launched.
int dispatch_host_direct(TagState& t, int n_walk, const std::vector<int32_t>& ord, const std::vector<Slot3>& off,
                         const std::vector<SplitPlan>& plan, int n_desc, const void* const* epi, const int* n_epi,
                         const pgf_epi_layout* il, const int* const* id_epj, const int* n_epj,
                         const int* const* id_spj, const int* n_spj, bool co_mode, bool gr_mode, double t0) {
    PGF_CUDA(t.h_src.ensure(n_walk));
    PGF_CUDA(t.h_hd_err.ensure(2));
    std::vector<int> plan_of(n_walk, -1);
    for (size_t q = 0; q < plan.size(); ++q) plan_of[plan[q].k] = (int)q;
    std::vector<std::pair<double, int>> cq(n_desc);
    for (int k = 0; k < n_walk; ++k) {
        const int w = ord[k];
        WalkSrc ws;
        ws.epi = static_cast<const char*>(epi[w]);
        ws.id_epj = n_epj[w] ? id_epj[w] : nullptr;
        ws.id_spj = n_spj[w] ? id_spj[w] : nullptr;
        ws.i_off = off[k].i;
        ws.e_off = off[k].e;
        ws.s_off = off[k].s;
        ws.rcut2 = g.walk_rcut2.empty() ? g.rcut2 : g.walk_rcut2[w];
        ws.n_i = n_epi[w];
        ws.n_epj = n_epj[w];
        ws.n_spj = n_spj[w];
        ws.walk = w;
        ws.parts = 1;
        ws.desc1 = 0;
        ws.rows1 = 0;
        ws.split = -1;
        ws.pad = 0;
        if (plan_of[k] >= 0) {
            const SplitPlan& sp = plan[plan_of[k]];
            ws.parts = sp.parts;
            ws.desc1 = sp.desc1;
            ws.rows1 = sp.rows1;
            ws.split = plan_of[k];
            for (int j = 1; j < sp.parts; ++j)
                cq[sp.desc1 + j - 1] = {part_cost(n_epi[w], n_epj[w], n_spj[w], j, sp.parts), sp.desc1 + j - 1};
        }
        cq[k] = {part_cost(n_epi[w], n_epj[w], n_spj[w], 0, ws.parts), k};
        t.h_src.h[k] = ws;
    }
    if (plan.empty()) {
        for (int k = 0; k < n_desc; ++k) t.h_order.h[k] = k;
    } else {
        queue_order(cq, t.h_order.h);
        PGF_CUDA(t.splits.ensure(plan.size()));
    }
    // The gather reads the walk table and the order from pinned host memory
    // in place and writes the split records itself.
    HdWalkArgs a{};
    a.src = t.h_src.h;
    a.n_walk = n_walk;
    a.n_desc = n_desc;
    a.order_src = t.h_order.h;
    a.order_dst = t.order.d;
    a.out_splits = plan.empty() ? nullptr : t.splits.d;
    a.epi_size = il->size;
    a.epi_off_pos = il->off_pos;
    a.epi_off_rs = il->off_r_search;
    if (gr_mode) {
        a.gr_epi_off_acc = g.gr.epi_off_acc;
        a.out_epi_acc = t.epi_acc.d;
    }
    if (co_mode) {
        a.co_epi_off_id = g.co.epi_off_id;
        a.co_epi_off_r_in = g.co.epi_off_r_in;
        a.co_epi_off_r_out = g.co.epi_off_r_out;
        a.co_epi_off_self_mass = g.co.epi_off_self_mass;
        a.out_epi_co = t.epi_co.d;
    }
    a.n_epj_tot = g.n_epj_tot;
    a.n_spj_tot = g.n_spj_tot;
    a.out_epi = t.epi.d;
    a.out_id_epj = t.id_epj.d;
    a.out_id_spj = t.id_spj.d;
    a.out_walks = t.walks.d;
    const int tag = (int)(&t - g.tags);
    a.err = g.hd_err.d + kHdErrWords * tag;
    a.err_host = t.h_hd_err.h;
    g.prof.copy += now_s() - t0;
    PGF_CUDA(cudaEventRecord(t.ev[0], g.stream));
    {
        const cudaError_t e = launch_gather_walks(a, g.num_sms, g.stream);
        if (e != cudaSuccess) return fail(PGF_ERR_CUDA, "walk gather kernel failed: %s", cudaGetErrorString(e));
    }
    PGF_CUDA(cudaEventRecord(t.ev_in, g.stream));
    // The force kernels are queued right behind the gather, with no host
    // round trip between: they read the check's outcome themselves and run
    // nothing when an id was out of range.
    t.params.input_err = a.err + 3;
    t.n_split = (int)plan.size();
    if (int r = launch_tag(t)) return r;
    // The caller's arrays are only valid during the call: return once the
    // gather has read them, with the check's outcome.
    PGF_CUDA(cudaEventSynchronize(t.ev_in));
    if (t.h_hd_err.h[0] != 0) {
        t.dispatched = false;
        t.has_data = false;
        return fail(PGF_ERR_ARG, "walk %d has an EPJ/SPJ id outside the sent arrays", t.h_hd_err.h[1]);
    }
    return PGF_OK;
}

// Packs the walks of one index dispatch (src/force_gpu_cuda.cu:621-699) and
// launches the kernels.  Walks are laid out in descending cost (EP-SP pairs
// weighted by their larger instruction count), so the work queue is the
// identity and the largest walks start first.  Large dispatches run as a
// pipeline of up to kMaxChunks stages over contiguous ranges of that layout:
// the host packs stage c + 1 while the copy stream moves stage c, and each
// stage's kernels run on their own stream as soon as its copies land, so a
// stage's tail overlaps the next stage's start.
int dispatch_walks(int tag, int n_walk, const void* const* epi, const int* n_epi, const pgf_epi_layout* il,
                   const int* const* id_epj, const int* n_epj, const int* const* id_spj, const int* n_spj) {
    TagState& t = g.tags[tag];
    if (n_walk < 0) return fail(PGF_ERR_ARG, "n_walk < 0");
    if (n_walk > 0 && (!epi || !n_epi || !il || !n_epj || !n_spj))
        return fail(PGF_ERR_ARG, "walk arrays or EPI layout are NULL");
    if (!g.walk_rcut2.empty() && (int)g.walk_rcut2.size() != n_walk)
        return fail(PGF_ERR_ARG, "per-walk r_out^2 was set for %zu walks, dispatch has %d",
                    g.walk_rcut2.size(), n_walk);
    // Earlier work of this tag may still read its staging or device buffers.
    if (t.dispatched) PGF_CUDA(cudaEventSynchronize(t.ev[3]));
    const double t0 = now_s();
    for (int w = 0; w < n_walk; ++w) {
        if (n_epi[w] < 0 || n_epj[w] < 0 || n_spj[w] < 0) return fail(PGF_ERR_ARG, "negative count in walk %d", w);
        if ((n_epi[w] > 0 && !epi[w]) || (n_epj[w] > 0 && (!id_epj || !id_epj[w])) ||
            (n_spj[w] > 0 && (!id_spj || !id_spj[w])))
            return fail(PGF_ERR_ARG, "NULL array for walk %d", w);
    }
    auto cost = [&](int w) { return (double)n_epi[w] * ((double)n_epj[w] + 2.0 * (double)n_spj[w]); };
    // Descending cost, ties in walk order (the order a stable sort gives),
    // with the costs computed once.
    std::vector<std::pair<double, int32_t>> by_cost(n_walk);
    for (int w = 0; w < n_walk; ++w) by_cost[w] = {cost(w), w};
    std::sort(by_cost.begin(), by_cost.end(), [](const std::pair<double, int32_t>& a, const std::pair<double, int32_t>& b) {
        return a.first > b.first || (a.first == b.first && a.second < b.second);
    });
    std::vector<int32_t> ord(n_walk);
    for (int k = 0; k < n_walk; ++k) ord[k] = by_cost[k].second;
    std::vector<Slot3> off(n_walk + 1);
    off[0] = Slot3{0, 0, 0};
    t.epi_disp.assign(n_walk, 0);
    for (int k = 0; k < n_walk; ++k) {
        const int w = ord[k];
        t.epi_disp[w] = off[k].i;
        off[k + 1] = Slot3{off[k].i + n_epi[w], off[k].e + n_epj[w], off[k].s + n_spj[w]};
    }
    const int64_t ni = off[n_walk].i, ne = off[n_walk].e, ns = off[n_walk].s;
    if (ni > kMaxRows) return fail(PGF_ERR_CAPACITY, "%lld i-particles exceed 2^31-1", (long long)ni);
    if (ne > 0 && !g.j_sent) return fail(PGF_ERR_STATE, "EPJ ids given before the EPJ array was sent");
    const bool co_mode = g.mode == PGF_MODE_FORCE_CHANGEOVER;
    if (co_mode && !g.co_set) return fail(PGF_ERR_STATE, "changeover mode without pgf_set_changeover_layout");
    if (co_mode && ne > 0 && !g.j_co_sent)
        return fail(PGF_ERR_STATE, "changeover mode: the EPJ array was sent before the changeover layout was set");
    const bool gr_mode = g.mode == PGF_MODE_GRADIENT;
    if (gr_mode && !g.gr_set) return fail(PGF_ERR_STATE, "gradient mode without pgf_set_gradient_layout");
    if (gr_mode && ne > 0 && !g.j_gr_sent)
        return fail(PGF_ERR_STATE, "gradient mode: the EPJ array was sent before the gradient layout was set");
    t.mode = g.mode;
    // Stages: contiguous ranges of the sorted layout.  The first has a quarter
    // of the list entries of the others, so the GPU starts sooner; the rest
    // share the remainder equally.
    int n_chunks = g.stages > 0 ? g.stages : (int)std::min<int64_t>(kMaxChunks, (ne + ns) / kChunkIdEntries + 1);
    if (n_walk < 8 * n_chunks) n_chunks = 1;
    const bool hd_single =
        n_chunks == 1 && use_hd() && hd_walks_ok(n_walk, epi, n_epi, il, id_epj, n_epj, id_spj, n_spj, t.mode);

    // Split plan.  In a single launch the most expensive walks bound the
    // launch time when there are few walks per CTA.  The unit is a sixteenth
    // of one SM's even share of the dispatch's cost; each walk that costs
    // more than a unit runs as parts of at most a unit (at most 16 parts, at
    // least 256 list entries each), each with a slice of its EPJ and SPJ
    // lists and its own copy of the walk's EPI rows (made on the device), and
    // a combine kernel adds the parts up.  The kernels add per-i terms
    // (changeover self-potential, the gradient pass's a_i) in part 0 only.
    // On 200-walk batches of the 1M binary Plummer workload an eighth ran
    // the kernels 24% faster than parts of a quarter share split only above
    // two units, and a sixteenth another 5% faster than an eighth.
    std::vector<SplitPlan> plan;
    int64_t ni_all = ni;
    int n_desc = n_walk;
    if (n_chunks == 1 && g.walk_split && n_walk > 0) {
        double total = 0.0;
        for (int k = 0; k < n_walk; ++k) total += cost(ord[k]);
        const double target = total / ((double)g.split_div * (double)g.num_sms);
        for (int k = 0; k < n_walk; ++k) {
            const int w = ord[k];
            const double c = cost(w);
            if (!(c > target)) break;  // the layout is sorted by cost
            const int64_t entries = (int64_t)n_epj[w] + n_spj[w];
            const int parts = (int)std::min<double>({16.0, std::ceil(c / target), (double)(entries / 256)});
            if (parts < 2) continue;
            plan.push_back(SplitPlan{k, parts, ni_all, n_desc});
            ni_all += (int64_t)(parts - 1) * n_epi[w];
            n_desc += parts - 1;
        }
        if (ni_all > kMaxRows) {
            plan.clear();
            ni_all = ni;
            n_desc = n_walk;
        }
    }
    t.n_split = 0;
    if (gr_mode) {
        if (!hd_single) PGF_CUDA(t.h_epi_acc.ensure(ni));
        PGF_CUDA(t.epi_acc.ensure(ni_all));
        PGF_CUDA(t.acorr.ensure(ni_all));
    }
    if (co_mode) {
        if (!hd_single) PGF_CUDA(t.h_epi_co.ensure(ni));
        PGF_CUDA(t.epi_co.ensure(ni_all));
        PGF_CUDA(t.pot_soft.ensure(ni_all));
    }

    if (!hd_single) {  // pinned staging of the host packing
        PGF_CUDA(t.h_epi.ensure(ni));
        PGF_CUDA(t.h_id_epj.ensure(ne));
        PGF_CUDA(t.h_id_spj.ensure(ns));
        PGF_CUDA(t.h_walks.ensure(n_desc));
    }
    PGF_CUDA(t.h_order.ensure(n_desc));
    PGF_CUDA(t.epi.ensure(ni_all));
    PGF_CUDA(t.id_epj.ensure(ne));
    PGF_CUDA(t.id_spj.ensure(ns));
    PGF_CUDA(t.walks.ensure(n_desc));
    PGF_CUDA(t.order.ensure(n_desc));
    PGF_CUDA(t.accp.ensure(ni_all));
    PGF_CUDA(t.nnb.ensure(ni_all));
    std::vector<int> cb(n_chunks + 1, n_walk);
    cb[0] = 0;
    for (int c = 1, k = 0; c < n_chunks; ++c) {
        const int64_t target = (ne + ns) * (4 * c - 3) / (4 * n_chunks - 3);
        while (k < n_walk && off[k].e + off[k].s < target) ++k;
        cb[c] = k;
    }

    t.n_walk = n_walk;
    t.ni_tot = ni;
    t.n_epi.assign(n_epi, n_epi + n_walk);
    t.precision = g.precision;
    t.variant = g.variant;
    Params& p = t.params;
    p = Params{};
    p.epi = t.epi.d;
    p.epj = g.epj.d;
    p.epj_m64 = g.epj_m64.d;
    p.epj_rs64 = g.epj_rs64.d;
    p.spj = g.spj.d;
    p.spj_q64 = g.spj_q64.d;
    p.epj32 = g.epj32.d;
    p.spj32 = g.spj32.d;
    if (gr_mode) {
        p.epj_acc32 = g.epj_acc32.d;
        p.epi_acc64 = t.epi_acc.d;
        p.out_acorr = t.acorr.d;
    }
    if (co_mode) {
        p.epj_co = g.epj_co.d;
        p.epi_co = t.epi_co.d;
        p.out_pot_soft = t.pot_soft.d;
    }
    p.id_epj = t.id_epj.d;
    p.id_spj = t.id_spj.d;
    p.walks = t.walks.d;
    p.order = t.order.d;
    p.n_walk = n_desc;
    p.gr_compensated = g.gr_compensated;
    // The neighbour search tests r^2 < max(rs_i, rs_j)^2 without softening
    // (src/soft_force.hpp:11-34); the force kernels include eps^2.
    p.eps2 = t.mode == PGF_MODE_NEIGHBOR_SEARCH ? 0.0 : g.eps2;
    p.G = g.G;
    p.out_accp = t.accp.d;
    p.out_nnb = t.nnb.d;
    bind_scratch(p);
    g.prof.n_walk += n_walk;
    g.prof.n_epi += ni;
    g.prof.n_epj += ne;
    g.prof.n_spj += ns;
    g.prof.n_call += 1;

    // One walk per task: the layout is in descending cost, so larger chunks
    // would give one thread the largest walks of a small dispatch.
    auto pack_range = [&](int k0, int k1) -> int {
        int bad_walk = -1;
#pragma omp parallel for schedule(dynamic, 1) reduction(max : bad_walk)
        for (int k = k0; k < k1; ++k)
            if (!pack_walk(t, k, ord[k], off[k], epi, n_epi, il, id_epj, n_epj, id_spj, n_spj))
                bad_walk = std::max(bad_walk, ord[k]);
        return bad_walk;
    };
    // Host-to-device copies of layout positions [k0, k1) on stream s.
    auto copy_range = [&](int k0, int k1, cudaStream_t s) -> int {
        const Slot3 a = off[k0], b = off[k1];
        if (b.i > a.i)
            PGF_CUDA(cudaMemcpyAsync(t.epi.d + a.i, t.h_epi.h + a.i, (b.i - a.i) * sizeof(EpiDev),
                                     cudaMemcpyHostToDevice, s));
        if (b.i > a.i && gr_mode)
            PGF_CUDA(cudaMemcpyAsync(t.epi_acc.d + a.i, t.h_epi_acc.h + a.i, (b.i - a.i) * sizeof(Accp),
                                     cudaMemcpyHostToDevice, s));
        if (b.i > a.i && co_mode)
            PGF_CUDA(cudaMemcpyAsync(t.epi_co.d + a.i, t.h_epi_co.h + a.i, (b.i - a.i) * sizeof(CoRec),
                                     cudaMemcpyHostToDevice, s));
        if (b.e > a.e)
            PGF_CUDA(cudaMemcpyAsync(t.id_epj.d + a.e, t.h_id_epj.h + a.e, (b.e - a.e) * sizeof(int32_t),
                                     cudaMemcpyHostToDevice, s));
        if (b.s > a.s)
            PGF_CUDA(cudaMemcpyAsync(t.id_spj.d + a.s, t.h_id_spj.h + a.s, (b.s - a.s) * sizeof(int32_t),
                                     cudaMemcpyHostToDevice, s));
        if (k1 > k0) {
            PGF_CUDA(cudaMemcpyAsync(t.walks.d + k0, t.h_walks.h + k0, (k1 - k0) * sizeof(WalkDesc),
                                     cudaMemcpyHostToDevice, s));
            PGF_CUDA(cudaMemcpyAsync(t.order.d + k0, t.h_order.h + k0, (k1 - k0) * sizeof(int32_t),
                                     cudaMemcpyHostToDevice, s));
        }
        return PGF_OK;
    };

    if (hd_single) {
        t.ord = ord;
        return dispatch_host_direct(t, n_walk, ord, off, plan, n_desc, epi, n_epi, il, id_epj, n_epj, id_spj, n_spj,
                                    co_mode, gr_mode, t0);
    }
    if (n_chunks == 1) {
        t.ord = ord;
        const int bad_walk = pack_range(0, n_walk);
        if (bad_walk >= 0) {
            g.prof.copy += now_s() - t0;
            return fail(PGF_ERR_ARG, "walk %d has an EPJ/SPJ id outside the sent arrays", bad_walk);
        }
        if (!plan.empty()) {
            PGF_CUDA(t.h_splits.ensure(plan.size()));
            PGF_CUDA(t.splits.ensure(plan.size()));
            for (size_t q = 0; q < plan.size(); ++q) {
                const SplitPlan& sp = plan[q];
                const WalkDesc d0 = t.h_walks.h[sp.k];
                for (int j = 0; j < sp.parts; ++j) {
                    WalkDesc d = d0;
                    const int e0 = (int)((int64_t)d0.n_epj * j / sp.parts);
                    const int e1 = (int)((int64_t)d0.n_epj * (j + 1) / sp.parts);
                    const int s0 = (int)((int64_t)d0.n_spj * j / sp.parts);
                    const int s1 = (int)((int64_t)d0.n_spj * (j + 1) / sp.parts);
                    d.epj_begin = d0.epj_begin + e0;
                    d.n_epj = e1 - e0;
                    d.spj_begin = d0.spj_begin + s0;
                    d.n_spj = s1 - s0;
                    if (j == 0) {
                        t.h_walks.h[sp.k] = d;
                        continue;
                    }
                    // Part j reads a copy of the walk's rows, made on the
                    // device after the copies (launch_split_rows).
                    d.i_begin = (int32_t)(sp.rows1 + (int64_t)(j - 1) * d0.n_i);
                    d.part = j;
                    t.h_walks.h[sp.desc1 + j - 1] = d;
                }
                t.h_splits.h[q] = SplitRec{d0.i_begin, (int32_t)sp.rows1, d0.n_i, sp.parts};
            }
            // Work queue over walks and parts, by descending cost.
            std::vector<std::pair<double, int>> cq(n_desc);
            for (int k = 0; k < n_desc; ++k) {
                const WalkDesc& d = t.h_walks.h[k];
                cq[k] = {(double)d.n_i * ((double)d.n_epj + 2.0 * (double)d.n_spj), k};
            }
            queue_order(cq, t.h_order.h);
        }
        g.prof.copy += now_s() - t0;
        PGF_CUDA(cudaEventRecord(t.ev[0], g.stream));
        if (int r = copy_range(0, n_walk, g.stream)) return r;
        if (!plan.empty()) {
            PGF_CUDA(cudaMemcpyAsync(t.walks.d, t.h_walks.h, n_desc * sizeof(WalkDesc), cudaMemcpyHostToDevice,
                                     g.stream));
            PGF_CUDA(cudaMemcpyAsync(t.order.d, t.h_order.h, n_desc * sizeof(int32_t), cudaMemcpyHostToDevice,
                                     g.stream));
            PGF_CUDA(cudaMemcpyAsync(t.splits.d, t.h_splits.h, plan.size() * sizeof(SplitRec),
                                     cudaMemcpyHostToDevice, g.stream));
            const cudaError_t e = launch_split_rows(t.splits.d, (int)plan.size(), t.epi.d, co_mode ? t.epi_co.d : nullptr,
                                                    gr_mode ? t.epi_acc.d : nullptr, g.stream);
            if (e != cudaSuccess) return fail(PGF_ERR_CUDA, "split rows kernel failed: %s", cudaGetErrorString(e));
            t.n_split = (int)plan.size();
        }
        return launch_tag(t);
    }

    // Pipelined stages.  The copy stream starts after everything already
    // queued on the compute stream (the EPJ/SPJ copies); the compute stream
    // resumes after every stage is done.
    cudaStream_t cs = g.copy_stream;
    auto drain = [&]() {
        cudaStreamSynchronize(cs);
        for (int c = 0; c < n_chunks; ++c) cudaStreamSynchronize(g.stage_stream[c]);
    };
    PGF_CUDA(cudaEventRecord(t.ev[0], g.stream));
    PGF_CUDA(cudaStreamWaitEvent(cs, t.ev[0], 0));
    double pack_s = now_s() - t0;
    for (int c = 0; c < n_chunks; ++c) {
        const int k0 = cb[c], k1 = cb[c + 1];
        const double tp = now_s();
        const int bad_walk = pack_range(k0, k1);
        pack_s += now_s() - tp;
        if (bad_walk >= 0) {
            // Stages already launched use valid data; let them finish before
            // the caller may touch the staging buffers again.
            drain();
            g.prof.copy += pack_s;
            return fail(PGF_ERR_ARG, "walk %d has an EPJ/SPJ id outside the sent arrays", bad_walk);
        }
        cudaStream_t sc = g.stage_stream[c];
        int r = PGF_OK;
        if (cudaEventRecord(t.evc[c][0], cs) != cudaSuccess || (r = copy_range(k0, k1, cs)) != PGF_OK ||
            cudaEventRecord(t.evc[c][1], cs) != cudaSuccess || cudaStreamWaitEvent(sc, t.evc[c][1], 0) != cudaSuccess) {
            drain();
            return r ? r : fail(PGF_ERR_CUDA, "pipelined copy of stage %d failed", c);
        }
        Params pc = p;
        pc.order = t.order.d + k0;
        pc.n_walk = k1 - k0;
        bind_scratch(pc, c, n_chunks);
        if ((r = launch_kernels(t, pc, sc, t.evc[c][2], t.evc[c][3])) != PGF_OK) {
            drain();
            return r;
        }
        if (cudaEventRecord(t.evc[c][4], sc) != cudaSuccess || cudaStreamWaitEvent(g.stream, t.evc[c][4], 0) != cudaSuccess) {
            drain();
            return fail(PGF_ERR_CUDA, "stage %d event failed", c);
        }
    }
    PGF_CUDA(cudaEventRecord(t.ev[3], g.stream));
    g.prof.copy += pack_s;
    t.ord = ord;
    t.stage_k = cb;
    t.stage_i.resize(n_chunks + 1);
    for (int c = 0; c <= n_chunks; ++c) t.stage_i[c] = off[cb[c]].i;
    t.n_chunks = n_chunks;
    t.dispatched = true;
    t.has_data = true;
    t.times_pending = true;
    return PGF_OK;
}

bool valid_tag(int tag) { return tag >= 0 && tag < kMaxTags; }

}  // namespace

extern "C" {

int pgf_initialize(int rank, double eps2, double rcut2, double G) {
    if (!(eps2 >= 0) || !(rcut2 >= 0) || !std::isfinite(G))
        return fail(PGF_ERR_ARG, "eps2 and rcut2 must be >= 0 and G finite");
    if (!g.init) {
        int r = setup_device(rank);
        if (r != PGF_OK) return r;
    } else {
        PGF_CUDA(cudaSetDevice(g.device));
    }
    g.eps2 = eps2;
    g.rcut2 = rcut2;
    g.G = G;
    g_error.clear();
    return PGF_OK;
}

int pgf_set_precision(int precision) {
    if (precision != PGF_PRECISION_MIXED && precision != PGF_PRECISION_FP64)
        return fail(PGF_ERR_ARG, "unknown precision %d", precision);
    g.precision = precision;
    return PGF_OK;
}

int pgf_set_stream(void* cuda_stream) {
    g.user_stream = cuda_stream != nullptr;
    g.stream = cuda_stream ? (cudaStream_t)cuda_stream : g.own_stream;
    return PGF_OK;
}

int pgf_set_walk_rcut2(const double* walk_rcut2, int n_walk) {
    if (n_walk < 0 || (n_walk > 0 && !walk_rcut2)) return fail(PGF_ERR_ARG, "bad per-walk r_out^2 array");
    for (int w = 0; w < n_walk; ++w)
        if (!(walk_rcut2[w] >= 0)) return fail(PGF_ERR_ARG, "per-walk r_out^2 must be >= 0");
    g.walk_rcut2.assign(walk_rcut2, walk_rcut2 + n_walk);
    return PGF_OK;
}

int pgf_dispatch_index(int tag, int n_walk, const void* const* epi, const int* n_epi,
                       const pgf_epi_layout* epi_layout, const int* const* id_epj, const int* n_epj,
                       const int* const* id_spj, const int* n_spj, const void* epj, int n_epj_tot,
                       const pgf_epj_layout* epj_layout, const void* spj, int n_spj_tot,
                       const pgf_spj_layout* spj_layout, int send_flag) {
    if (int r = ensure_init()) return r;
    if (!valid_tag(tag)) return fail(PGF_ERR_ARG, "tag %d outside [0, %d)", tag, kMaxTags);
    PGF_CUDA(cudaSetDevice(g.device));
    if (send_flag) return pack_and_send_j(epj, n_epj_tot, epj_layout, spj, n_spj_tot, spj_layout);
    return dispatch_walks(tag, n_walk, epi, n_epi, epi_layout, id_epj, n_epj, id_spj, n_spj);
}

int pgf_dispatch(int tag, int n_walk, const void* const* epi, const int* n_epi, const pgf_epi_layout* epi_layout,
                 const void* const* epj, const int* n_epj, const pgf_epj_layout* epj_layout,
                 const void* const* spj, const int* n_spj, const pgf_spj_layout* spj_layout) {
    if (int r = ensure_init()) return r;
    if (!valid_tag(tag)) return fail(PGF_ERR_ARG, "tag %d outside [0, %d)", tag, kMaxTags);
    if (n_walk < 0) return fail(PGF_ERR_ARG, "n_walk < 0");
    if (n_walk > 0 && (!n_epj || !n_spj)) return fail(PGF_ERR_ARG, "per-walk counts are NULL");
    PGF_CUDA(cudaSetDevice(g.device));
    // The per-walk j arrays are concatenated into the shared arrays and
    // addressed through identity id lists.
    int64_t ne = 0, ns = 0;
    for (int w = 0; w < n_walk; ++w) {
        if (n_epj[w] < 0 || n_spj[w] < 0) return fail(PGF_ERR_ARG, "negative count in walk %d", w);
        if ((n_epj[w] > 0 && (!epj || !epj[w] || !epj_layout)) || (n_spj[w] > 0 && (!spj || !spj[w] || !spj_layout)))
            return fail(PGF_ERR_ARG, "NULL j array for walk %d", w);
        ne += n_epj[w];
        ns += n_spj[w];
    }
    if (ne > kMaxRows || ns > kMaxRows) return fail(PGF_ERR_CAPACITY, "j rows exceed 2^31-1");
    std::vector<char> ej(ne * sizeof(double) * 5), sj(ns * sizeof(double) * 10);
    std::vector<int> ids_e(ne), ids_s(ns);
    std::vector<const int*> pe(n_walk), ps(n_walk);
    int64_t oe = 0, os = 0;
    for (int w = 0; w < n_walk; ++w) {
        for (int k = 0; k < n_epj[w]; ++k) {
            const char* r = reinterpret_cast<const char*>(epj[w]) + (size_t)k * epj_layout->size;
            double* o = reinterpret_cast<double*>(ej.data()) + 5 * (oe + k);
            const double* p = dptr(r, epj_layout->off_pos);
            o[0] = *dptr(r, epj_layout->off_mass);
            o[1] = p[0];
            o[2] = p[1];
            o[3] = p[2];
            o[4] = *dptr(r, epj_layout->off_r_search);
            ids_e[oe + k] = (int)(oe + k);
        }
        for (int k = 0; k < n_spj[w]; ++k) {
            const char* r = reinterpret_cast<const char*>(spj[w]) + (size_t)k * spj_layout->size;
            double* o = reinterpret_cast<double*>(sj.data()) + 10 * (os + k);
            const double* p = dptr(r, spj_layout->off_pos);
            o[0] = *dptr(r, spj_layout->off_mass);
            o[1] = p[0];
            o[2] = p[1];
            o[3] = p[2];
            for (int c = 0; c < 6; ++c) o[4 + c] = spj_layout->has_quad ? dptr(r, spj_layout->off_quad)[c] : 0.0;
            ids_s[os + k] = (int)(os + k);
        }
        pe[w] = ids_e.data() + oe;
        ps[w] = ids_s.data() + os;
        oe += n_epj[w];
        os += n_spj[w];
    }
    const pgf_epj_layout el{5 * sizeof(double), 0, sizeof(double), 4 * sizeof(double)};
    const pgf_spj_layout sl{10 * sizeof(double), 0, sizeof(double), 4 * sizeof(double), 1};
    int r = pack_and_send_j(ej.data(), ne, &el, sj.data(), ns, &sl);
    if (r != PGF_OK) return r;
    return dispatch_walks(tag, n_walk, epi, n_epi, epi_layout, pe.data(), n_epj, ps.data(), n_spj);
}

int pgf_recompute(int tag) {
    if (int r = ensure_init()) return r;
    if (!valid_tag(tag)) return fail(PGF_ERR_ARG, "tag %d outside [0, %d)", tag, kMaxTags);
    TagState& t = g.tags[tag];
    if (!t.has_data) return fail(PGF_ERR_STATE, "tag %d has no dispatched data", tag);
    PGF_CUDA(cudaSetDevice(g.device));
    PGF_CUDA(cudaEventRecord(t.ev[0], g.stream));
    t.precision = g.precision;
    t.variant = g.variant;
    return launch_tag(t);
}

int pgf_set_kernel_variant(int variant) {
    if (variant < 0 || variant >= PGF_NUM_KERNEL_VARIANTS)
        return fail(PGF_ERR_ARG, "kernel variant %d outside [0, %d)", variant, PGF_NUM_KERNEL_VARIANTS);
    g.variant = variant;
    return PGF_OK;
}

int pgf_set_mode(int mode) {
    if (mode != PGF_MODE_FORCE && mode != PGF_MODE_NEIGHBOR_SEARCH && mode != PGF_MODE_FORCE_CHANGEOVER &&
        mode != PGF_MODE_GRADIENT)
        return fail(PGF_ERR_ARG, "unknown mode %d", mode);
    g.mode = mode;
    return PGF_OK;
}

int pgf_set_gradient_layout(const pgf_gradient_layout* layout) {
    if (!layout) {
        g.gr_set = false;
        return PGF_OK;
    }
    g.gr = *layout;
    g.gr_set = true;
    return PGF_OK;
}

int pgf_set_changeover_layout(const pgf_changeover_layout* layout) {
    if (!layout) {
        g.co_set = false;
        return PGF_OK;
    }
    g.co = *layout;
    g.co_set = true;
    return PGF_OK;
}

int pgf_set_wait_limit_ns(uint64_t limit_ns) {
    g.wait_limit_ns = limit_ns;
    return PGF_OK;
}

int pgf_test_stall_producer(int items) {
    if (items < 0) return fail(PGF_ERR_ARG, "items must be >= 0");
    g.stall_after_items = items;
    return PGF_OK;
}

int pgf_set_host_direct(int enable) {
    g.hd_enabled = enable != 0;
    return PGF_OK;
}

int pgf_get_host_direct(int* active) {
    if (!active) return fail(PGF_ERR_ARG, "NULL argument");
    *active = use_hd() ? 1 : 0;
    return PGF_OK;
}

int pgf_set_walk_split(int enable) {
    g.walk_split = enable != 0;
    return PGF_OK;
}

int pgf_set_gradient_accuracy(int mode) {
    if (mode != 0 && mode != 1) return fail(PGF_ERR_ARG, "gradient accuracy mode %d is not 0 or 1", mode);
    g.gr_compensated = mode;
    return PGF_OK;
}

int pgf_set_walk_split_unit(int div) {
    if (div < 1 || div > 256) return fail(PGF_ERR_ARG, "split unit divisor %d outside [1, 256]", div);
    g.split_div = div;
    return PGF_OK;
}

int pgf_set_dispatch_stages(int stages) {
    if (stages < 0 || stages > kMaxChunks)
        return fail(PGF_ERR_ARG, "dispatch stages %d outside [0, %d]", stages, kMaxChunks);
    g.stages = stages;
    return PGF_OK;
}

int pgf_get_kernel_variant(int* variant) {
    if (!variant) return fail(PGF_ERR_ARG, "NULL variant");
    *variant = g.variant;
    return PGF_OK;
}

int pgf_autotune(int tag, int repeats, int* best_variant, double* best_ms) {
    if (int r = ensure_init()) return r;
    if (!valid_tag(tag)) return fail(PGF_ERR_ARG, "tag %d outside [0, %d)", tag, kMaxTags);
    TagState& t = g.tags[tag];
    if (!t.has_data) return fail(PGF_ERR_STATE, "autotune needs a dispatched tag");
    if (repeats < 1) repeats = 1;
    PGF_CUDA(cudaSetDevice(g.device));
    const int saved_precision = g.precision;
    g.precision = PGF_PRECISION_MIXED;
    int best = g.variant;
    double best_t = HUGE_VAL;
    for (int v = 0; v < PGF_NUM_KERNEL_VARIANTS; ++v) {
        g.variant = v;
        double sum = 0.0;
        for (int k = 0; k <= repeats; ++k) {  // the first run warms up
            int r = pgf_recompute(tag);
            if (r == PGF_OK) r = pgf_wait(tag);
            if (r != PGF_OK) {
                g.precision = saved_precision;
                return r;
            }
            if (k > 0) sum += g.prof.last_calc_main;
        }
        if (sum < best_t) {
            best_t = sum;
            best = v;
        }
    }
    g.variant = best;
    g.precision = saved_precision;
    if (best_variant) *best_variant = best;
    if (best_ms) *best_ms = 1e3 * best_t / repeats;
    return PGF_OK;
}

int pgf_autotune_dispatch(int tag, int n_walk, const void* const* epi, const int* n_epi,
                          const pgf_epi_layout* epi_layout, const int* const* id_epj, const int* n_epj,
                          const int* const* id_spj, const int* n_spj, void* const* force,
                          const pgf_force_layout* force_layout, int repeats, int* best_stages, int* best_split,
                          double* best_ms) {
    if (int r = ensure_init()) return r;
    if (!valid_tag(tag)) return fail(PGF_ERR_ARG, "tag %d outside [0, %d)", tag, kMaxTags);
    if (repeats < 1) repeats = 1;
    const int saved_stages = g.stages, saved_div = g.split_div;
    struct Cand {
        int stages, div;
    };
    std::vector<Cand> cands;
    for (int st : {1, 2, 4, 8}) cands.push_back({st, g.split_div});
    for (int dv : {4, 8, 32}) cands.push_back({1, dv});
    double best_t = HUGE_VAL;
    Cand best{saved_stages, saved_div};
    for (const Cand& c : cands) {
        g.stages = c.stages;
        g.split_div = c.div;
        double t_min = HUGE_VAL;
        for (int k = 0; k <= repeats; ++k) {  // the first run warms up
            const double t0 = now_s();
            int r = pgf_dispatch_index(tag, n_walk, epi, n_epi, epi_layout, id_epj, n_epj, id_spj, n_spj, nullptr, 0,
                                       nullptr, nullptr, 0, nullptr, 0);
            if (r == PGF_OK) r = pgf_retrieve(tag, n_walk, n_epi, force, force_layout);
            if (r != PGF_OK) {
                g.stages = saved_stages;
                g.split_div = saved_div;
                return r;
            }
            if (k > 0) t_min = std::min(t_min, now_s() - t0);
        }
        if (t_min < best_t) {
            best_t = t_min;
            best = c;
        }
    }
    g.stages = best.stages;
    g.split_div = best.div;
    if (best_stages) *best_stages = best.stages;
    if (best_split) *best_split = best.div;
    if (best_ms) *best_ms = 1e3 * best_t;
    return PGF_OK;
}

// Writes the results of walk w into the caller's records.
void unpack_walk(const TagState& t, int w, const int* ni, void* const* force, const pgf_force_layout* fl) {
    char* base = reinterpret_cast<char*>(force[w]);
    const int64_t o = t.epi_disp[w];
    for (int i = 0; i < ni[w]; ++i) {
        char* r = base + (size_t)i * fl->size;
        if (t.mode != PGF_MODE_NEIGHBOR_SEARCH) {
            const Accp a = t.h_accp.h[o + i];
            double* acc = reinterpret_cast<double*>(r + fl->off_acc);
            acc[0] = a.x;
            acc[1] = a.y;
            acc[2] = a.z;
            *reinterpret_cast<double*>(r + fl->off_pot) = a.w;
            if (t.mode == PGF_MODE_FORCE_CHANGEOVER)
                *reinterpret_cast<double*>(r + g.co.force_off_pot_soft) = t.h_pot_soft.h[o + i];
            if (t.mode == PGF_MODE_GRADIENT) {
                double* ac = reinterpret_cast<double*>(r + g.gr.force_off_acorr);
                const Accp c = t.h_acorr.h[o + i];
                ac[0] = c.x;
                ac[1] = c.y;
                ac[2] = c.z;
            }
        }
        if (fl->n_ngb_bytes == 8)
            *reinterpret_cast<int64_t*>(r + fl->off_n_ngb) = t.h_nnb.h[o + i];
        else
            *reinterpret_cast<int32_t*>(r + fl->off_n_ngb) = t.h_nnb.h[o + i];
    }
}

// D2H copies of the result rows [r0, r1) on stream s.
int copy_back(TagState& t, int64_t r0, int64_t r1, cudaStream_t s) {
    if (r1 <= r0) return PGF_OK;
    const int64_t n = r1 - r0;
    PGF_CUDA(cudaMemcpyAsync(t.h_accp.h + r0, t.accp.d + r0, n * sizeof(Accp), cudaMemcpyDeviceToHost, s));
    PGF_CUDA(cudaMemcpyAsync(t.h_nnb.h + r0, t.nnb.d + r0, n * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    if (t.mode == PGF_MODE_GRADIENT)
        PGF_CUDA(cudaMemcpyAsync(t.h_acorr.h + r0, t.acorr.d + r0, n * sizeof(Accp), cudaMemcpyDeviceToHost, s));
    if (t.mode == PGF_MODE_FORCE_CHANGEOVER)
        PGF_CUDA(cudaMemcpyAsync(t.h_pot_soft.h + r0, t.pot_soft.d + r0, n * sizeof(double), cudaMemcpyDeviceToHost,
                                 s));
    return PGF_OK;
}

// Retrieve host-direct (single-launch dispatches): a scatter kernel writes
// each walk's results into the caller's Force records, so nothing is copied
// back or unpacked on the host.
int retrieve_host_direct(TagState& t, int n_walk, const int* ni, void* const* force, const pgf_force_layout* fl) {
    PGF_CUDA(t.h_dst.ensure(n_walk));
    for (int k = 0; k < n_walk; ++k) {
        const int w = t.ord[k];
        t.h_dst.h[k] = ForceDst{static_cast<char*>(force[w]), t.epi_disp[w], ni[w], 0};
    }
    HdScatterArgs a{};
    a.counts_only = t.mode == PGF_MODE_NEIGHBOR_SEARCH;
    a.size = fl->size;
    a.off_acc = fl->off_acc;
    a.off_pot = fl->off_pot;
    a.off_nnb = fl->off_n_ngb;
    a.nnb_bytes = fl->n_ngb_bytes;
    a.accp = t.accp.d;
    a.nnb = t.nnb.d;
    if (t.mode == PGF_MODE_FORCE_CHANGEOVER) {
        a.pot_soft = t.pot_soft.d;
        a.off_pot_soft = g.co.force_off_pot_soft;
    }
    if (t.mode == PGF_MODE_GRADIENT) {
        a.acorr = t.acorr.d;
        a.off_acorr = g.gr.force_off_acorr;
    }
    // The scatter reads the destination table from pinned host memory in
    // place and moves the status words into t.h_flags itself.
    a.dst = t.h_dst.h;
    a.n_walk = n_walk;
    a.flags_dev = g.scratch.d;
    a.flags_host = t.h_flags.h;
    cudaStream_t st = g.stream;
    PGF_CUDA(cudaEventRecord(t.ev[4], st));
    {
        const cudaError_t e = launch_scatter_results(a, g.num_sms, st);
        if (e != cudaSuccess) return fail(PGF_ERR_CUDA, "result scatter kernel failed: %s", cudaGetErrorString(e));
    }
    PGF_CUDA(cudaEventRecord(t.ev[5], st));
    PGF_CUDA(cudaEventSynchronize(t.ev[5]));
    t.dispatched = false;
    harvest_times(t);
    harvest_send();
    float ms_recv = 0;
    cudaEventElapsedTime(&ms_recv, t.ev[4], t.ev[5]);
    g.prof.recv += 1e-3 * ms_recv;
    g.prof.n_retest += t.h_flags.h[3];
    if (t.h_flags.h[2] != 0) return fail(PGF_ERR_DEVICE, "device error word %d", t.h_flags.h[2]);
    return PGF_OK;
}

int pgf_retrieve(int tag, int n_walk, const int* ni, void* const* force, const pgf_force_layout* fl) {
    if (int r = ensure_init()) return r;
    if (!valid_tag(tag)) return fail(PGF_ERR_ARG, "tag %d outside [0, %d)", tag, kMaxTags);
    TagState& t = g.tags[tag];
    if (!t.dispatched) return fail(PGF_ERR_STATE, "retrieve for tag %d without a dispatch", tag);
    if (n_walk != t.n_walk) return fail(PGF_ERR_ARG, "retrieve n_walk %d != dispatched %d", n_walk, t.n_walk);
    if (n_walk > 0 && (!ni || !force || !fl)) return fail(PGF_ERR_ARG, "NULL ni/force/layout");
    if (fl && fl->n_ngb_bytes != 4 && fl->n_ngb_bytes != 8) return fail(PGF_ERR_ARG, "n_ngb_bytes must be 4 or 8");
    for (int w = 0; w < n_walk; ++w) {
        if (ni[w] != t.n_epi[w]) return fail(PGF_ERR_ARG, "walk %d: ni %d != dispatched %d", w, ni[w], t.n_epi[w]);
        if (ni[w] > 0 && !force[w]) return fail(PGF_ERR_ARG, "force[%d] is NULL", w);
    }
    PGF_CUDA(cudaSetDevice(g.device));
    const int64_t n = t.ni_tot;
    PGF_CUDA(t.h_flags.ensure(4));
    // Host-direct results for single launches.  A pipelined dispatch keeps
    // the copy-engine copies and host unpacking per stage: those overlap the
    // later stages' kernels, where a scatter kernel would wait for their SMs.
    if (use_hd() && t.n_chunks == 0 && hd_force_ok(n_walk, ni, force, fl, t.mode))
        return retrieve_host_direct(t, n_walk, ni, force, fl);
    PGF_CUDA(t.h_accp.ensure(n));
    PGF_CUDA(t.h_nnb.ensure(n));
    if (t.mode == PGF_MODE_GRADIENT) PGF_CUDA(t.h_acorr.ensure(n));
    if (t.mode == PGF_MODE_FORCE_CHANGEOVER) PGF_CUDA(t.h_pot_soft.ensure(n));
    if (t.n_chunks > 0) {
        // Pipelined dispatch: copy back and unpack each stage as soon as its
        // kernels are done, while later stages still run.
        cudaStream_t ds = g.d2h_stream;
        for (int c = 0; c < t.n_chunks; ++c) {
            PGF_CUDA(cudaStreamWaitEvent(ds, t.evc[c][4], 0));
            if (c == 0) PGF_CUDA(cudaEventRecord(t.ev[4], ds));
            if (int r = copy_back(t, t.stage_i[c], t.stage_i[c + 1], ds)) return r;
            PGF_CUDA(cudaEventRecord(t.evc[c][5], ds));
        }
        // g.stream already waits for every stage; the flags follow them.
        PGF_CUDA(cudaStreamWaitEvent(ds, t.ev[3], 0));
        PGF_CUDA(cudaMemcpyAsync(t.h_flags.h, g.scratch.d, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, ds));
        PGF_CUDA(cudaMemsetAsync(g.scratch.d + 2, 0, 2 * sizeof(int32_t), ds));
        PGF_CUDA(cudaEventRecord(t.ev[5], ds));
        PGF_CUDA(cudaStreamWaitEvent(g.stream, t.ev[5], 0));  // later work follows the memset
        double unpack_s = 0.0;
        for (int c = 0; c < t.n_chunks; ++c) {
            PGF_CUDA(cudaEventSynchronize(t.evc[c][5]));
            const double t0 = now_s();
            const int k0 = t.stage_k[c], k1 = t.stage_k[c + 1];
#pragma omp parallel for schedule(dynamic, 8)
            for (int k = k0; k < k1; ++k) unpack_walk(t, t.ord[k], ni, force, fl);
            unpack_s += now_s() - t0;
        }
        PGF_CUDA(cudaEventSynchronize(t.ev[5]));
        t.dispatched = false;
        harvest_times(t);
        harvest_send();
        float ms_recv = 0;
        cudaEventElapsedTime(&ms_recv, t.ev[4], t.ev[5]);
        g.prof.recv += 1e-3 * ms_recv;
        g.prof.n_retest += t.h_flags.h[3];
        g.prof.copy += unpack_s;
        if (t.h_flags.h[2] != 0) return fail(PGF_ERR_DEVICE, "device error word %d", t.h_flags.h[2]);
        return PGF_OK;
    }
    cudaStream_t s = g.stream;
    PGF_CUDA(cudaEventRecord(t.ev[4], s));
    if (int r = copy_back(t, 0, n, s)) return r;
    PGF_CUDA(cudaMemcpyAsync(t.h_flags.h, g.scratch.d, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    PGF_CUDA(cudaMemsetAsync(g.scratch.d + 2, 0, 2 * sizeof(int32_t), s));
    PGF_CUDA(cudaEventRecord(t.ev[5], s));
    PGF_CUDA(cudaEventSynchronize(t.ev[5]));
    t.dispatched = false;
    harvest_times(t);
    harvest_send();
    float ms_recv = 0;
    cudaEventElapsedTime(&ms_recv, t.ev[4], t.ev[5]);
    g.prof.recv += 1e-3 * ms_recv;
    g.prof.n_retest += t.h_flags.h[3];
    if (t.h_flags.h[2] != 0) return fail(PGF_ERR_DEVICE, "device error word %d", t.h_flags.h[2]);
    const double t0 = now_s();
#pragma omp parallel for schedule(dynamic, 8)
    for (int w = 0; w < n_walk; ++w) unpack_walk(t, w, ni, force, fl);
    g.prof.copy += now_s() - t0;
    return PGF_OK;
}

int pgf_wait(int tag) {
    if (int r = ensure_init()) return r;
    if (!valid_tag(tag)) return fail(PGF_ERR_ARG, "tag %d outside [0, %d)", tag, kMaxTags);
    TagState& t = g.tags[tag];
    if (!t.has_data) return fail(PGF_ERR_STATE, "tag %d has no dispatched data", tag);
    PGF_CUDA(cudaSetDevice(g.device));
    PGF_CUDA(cudaEventSynchronize(t.ev[3]));
    harvest_times(t);
    harvest_send();
    return PGF_OK;
}

int pgf_get_profile(pgf_profile* out) {
    if (!out) return fail(PGF_ERR_ARG, "NULL profile");
    if (g.init) harvest_send();
    *out = g.prof;
    return PGF_OK;
}

int pgf_clear_profile(void) {
    g.prof = pgf_profile{};
    return PGF_OK;
}

const char* pgf_last_error(void) { return g_error.c_str(); }

int pgf_finalize(void) {
    if (!g.init) return PGF_OK;
    cudaSetDevice(g.device);
    cudaStreamSynchronize(g.stream);
    if (g.copy_stream) cudaStreamSynchronize(g.copy_stream);
    for (auto& st : g.stage_stream)
        if (st) cudaStreamSynchronize(st);
    if (g.d2h_stream) cudaStreamSynchronize(g.d2h_stream);
    for (auto& t : g.tags) {
        t.epi.release();
        t.id_epj.release();
        t.id_spj.release();
        t.order.release();
        t.walks.release();
        t.accp.release();
        t.nnb.release();
        t.h_epi.release();
        t.h_id_epj.release();
        t.h_id_spj.release();
        t.h_order.release();
        t.h_walks.release();
        t.h_accp.release();
        t.h_nnb.release();
        t.h_flags.release();
        t.epi_co.release();
        t.h_epi_co.release();
        t.pot_soft.release();
        t.h_pot_soft.release();
        t.epi_acc.release();
        t.h_epi_acc.release();
        t.acorr.release();
        t.h_acorr.release();
        t.splits.release();
        t.h_splits.release();
        t.h_src.release();
        t.h_dst.release();
        t.h_hd_err.release();
        if (t.ev_in) cudaEventDestroy(t.ev_in);
        t.ev_in = nullptr;
        for (auto& ev : t.ev) {
            if (ev) cudaEventDestroy(ev);
            ev = nullptr;
        }
        for (auto& c : t.evc)
            for (auto& ev : c) {
                if (ev) cudaEventDestroy(ev);
                ev = nullptr;
            }
        t.n_chunks = 0;
        t.dispatched = t.has_data = false;
    }
    g.epj.release();
    g.epj_m64.release();
    g.epj_rs64.release();
    g.spj.release();
    g.spj_q64.release();
    g.epj32.release();
    g.spj32.release();
    g.epj_co.release();
    g.h_epj_co.release();
    g.j_co_sent = false;
    g.epj_acc32.release();
    g.h_epj_acc32.release();
    g.j_gr_sent = false;
    g.h_epj.release();
    g.h_epj_m64.release();
    g.h_epj_rs64.release();
    g.h_spj.release();
    g.h_spj_q64.release();
    g.scratch.release();
    g.retest.release();
    g.hd_err.release();
    if (g.ev_send0) cudaEventDestroy(g.ev_send0);
    if (g.ev_send1) cudaEventDestroy(g.ev_send1);
    g.ev_send0 = g.ev_send1 = nullptr;
    if (g.own_stream) cudaStreamDestroy(g.own_stream);
    g.own_stream = nullptr;
    if (g.copy_stream) cudaStreamDestroy(g.copy_stream);
    g.copy_stream = nullptr;
    for (auto& st : g.stage_stream) {
        if (st) cudaStreamDestroy(st);
        st = nullptr;
    }
    if (g.d2h_stream) cudaStreamDestroy(g.d2h_stream);
    g.d2h_stream = nullptr;
    if (!g.user_stream) g.stream = nullptr;
    g.j_sent = false;
    g.init = false;
    return PGF_OK;
}

}  // extern "C"
