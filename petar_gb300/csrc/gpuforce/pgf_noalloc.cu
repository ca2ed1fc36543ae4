// Allocation-free entry point: the mixed-precision force evaluation on inputs
// and outputs that the caller already holds in device memory.
//
// Who needs it: host codes that own every byte of device memory themselves,
// for example a simulation that sizes one arena at start-up and hands out
// slices of it, or a time-stepping loop that cannot afford the device-wide
// synchronisation that cudaMalloc and cudaFree imply.  Such callers cannot let
// a library allocate on first use, as pgf_dispatch_index does.
//
// The interaction kernels need some scratch besides their inputs and outputs:
// per-walk descriptors (centre, box, largest r_search), the work-queue order,
// the queue cursor and the FP64 re-test records.  Here that scratch is the
// file-scope array g_noalloc_scratch, sized for PGF_NOALLOC_MAX_WALKS walks
// (about 2.6 MB); every GPU that loads the library keeps it until the process
// exits.  Host code cannot use the array's name as a device address: the first
// call on each device looks the address up with cudaGetSymbolAddress while
// that device is current, and later calls reuse it.
#include "petar_gpuforce.h"
#include "pgf_internal.cuh"

#include <cstdarg>
#include <cstddef>
#include <cstdio>

namespace {

using namespace pgf;

constexpr int kMaxWalks = PGF_NOALLOC_MAX_WALKS;
constexpr int kRetestCap = 1 << 16;
constexpr int kMaxDevices = 64;
constexpr size_t align256(size_t v) { return (v + 255) & ~size_t(255); }
constexpr size_t kFlagsOff = 0;  // [0] queue cursor, [1] re-test count, [2] error bits
constexpr size_t kDescOff = 256;
constexpr size_t kOrderOff = align256(kDescOff + sizeof(WalkDesc) * kMaxWalks);
constexpr size_t kRetestOff = align256(kOrderOff + sizeof(int32_t) * kMaxWalks);
constexpr size_t kScratchBytes = kRetestOff + sizeof(Retest) * kRetestCap;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

unsigned char* g_scratch_addr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

// Writes the message into the caller's buffer (if any) and returns the code.
int fail(char* buf, size_t len, int code, const char* fmt, ...) {
    if (buf && len) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, len, fmt, ap);
        va_end(ap);
    }
    return code;
}

static_assert(sizeof(pgf_epj_device) == sizeof(EpjMix), "pgf_epj_device must match EpjMix");
static_assert(sizeof(pgf_spj_device) == sizeof(SpjMix), "pgf_spj_device must match SpjMix");
static_assert(offsetof(pgf_epj_device, mass) == offsetof(EpjMix, m), "pgf_epj_device layout");
static_assert(offsetof(pgf_epj_device, r_search2) == offsetof(EpjMix, rs2), "pgf_epj_device layout");
static_assert(offsetof(pgf_spj_device, quad_traceless) == offsetof(SpjMix, Q), "pgf_spj_device layout");
static_assert(offsetof(pgf_spj_device, trace) == offsetof(SpjMix, tr), "pgf_spj_device layout");

enum : int { kBadWalk = 1, kBadEpjId = 2, kBadSpjId = 4 };

// One block per walk: checks the walk's table row and ids against the array
// sizes and fills its descriptor (box centre, half-extents and largest
// r_search rounded up, as the host packing of pgf_dispatch_index does).
__global__ __launch_bounds__(128) void walk_prep_kernel(int n_walk, const int64_t* table, const double* epi,
                                                        int64_t n_epi, int64_t n_epj, int64_t n_spj,
                                                        const int32_t* id_epj, int64_t n_id_epj,
                                                        const int32_t* id_spj, int64_t n_id_spj, double rcut2,
                                                        WalkDesc* desc, int32_t* order, int32_t* err) {
    __shared__ double red[7][128];
    __shared__ int bad;
    const int w = blockIdx.x;
    const int t = threadIdx.x;
    if (t == 0) bad = 0;
    __syncthreads();
    const int64_t* row = table + 6 * (int64_t)w;
    const int64_t i0 = row[0], ni = row[1], e0 = row[2], ne = row[3], s0 = row[4], ns = row[5];
    // Each range is tested as offset <= size - count with both terms
    // non-negative, so no sum can overflow whatever the table holds.
    const bool ok = ni >= 0 && ni <= 0x7fffffff && ni <= n_epi && i0 >= 0 && i0 <= n_epi - ni && ne >= 0 &&
                    ne <= 0x7fffffff && ne <= n_id_epj && e0 >= 0 && e0 <= n_id_epj - ne && ns >= 0 &&
                    ns <= 0x7fffffff && ns <= n_id_spj && s0 >= 0 && s0 <= n_id_spj - ns;
    if (!ok) {
        if (t == 0) atomicOr(err, kBadWalk);
        return;
    }
    for (int64_t k = t; k < ne; k += blockDim.x)
        if ((uint32_t)id_epj[e0 + k] >= (uint64_t)n_epj) atomicOr(&bad, kBadEpjId);
    for (int64_t k = t; k < ns; k += blockDim.x)
        if ((uint32_t)id_spj[s0 + k] >= (uint64_t)n_spj) atomicOr(&bad, kBadSpjId);
    double lo[3] = {HUGE_VAL, HUGE_VAL, HUGE_VAL}, hi[3] = {-HUGE_VAL, -HUGE_VAL, -HUGE_VAL}, rs = 0.0;
    for (int64_t i = t; i < ni; i += blockDim.x) {
        const double* e = epi + 4 * (i0 + i);
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], e[d]);
            hi[d] = fmax(hi[d], e[d]);
        }
        rs = fmax(rs, e[3]);
    }
    for (int d = 0; d < 3; ++d) {
        red[d][t] = lo[d];
        red[3 + d][t] = hi[d];
    }
    red[6][t] = rs;
    __syncthreads();
    for (int s = 64; s > 0; s >>= 1) {
        if (t < s) {
            for (int d = 0; d < 3; ++d) {
                red[d][t] = fmin(red[d][t], red[d][t + s]);
                red[3 + d][t] = fmax(red[3 + d][t], red[3 + d][t + s]);
            }
            red[6][t] = fmax(red[6][t], red[6][t + s]);
        }
        __syncthreads();
    }
    if (t == 0) {
        if (bad) atomicOr(err, bad);
        WalkDesc d;
        d.epj_begin = e0;
        d.spj_begin = s0;
        d.i_begin = (int32_t)i0;
        d.n_i = (int32_t)ni;
        d.n_epj = (int32_t)ne;
        d.n_spj = (int32_t)ns;
        if (ni > 0) {
            d.cx = 0.5 * (red[0][0] + red[3][0]);
            d.cy = 0.5 * (red[1][0] + red[4][0]);
            d.cz = 0.5 * (red[2][0] + red[5][0]);
            d.hx = __double2float_ru(fmax(red[3][0] - d.cx, d.cx - red[0][0]));
            d.hy = __double2float_ru(fmax(red[4][0] - d.cy, d.cy - red[1][0]));
            d.hz = __double2float_ru(fmax(red[5][0] - d.cz, d.cz - red[2][0]));
            d.rs_max = __double2float_ru(red[6][0]);
        } else {
            d.cx = d.cy = d.cz = 0.0;
            d.hx = d.hy = d.hz = d.rs_max = 0.f;
        }
        d.part = 0;
        d.pad[0] = d.pad[1] = d.pad[2] = 0.f;
        d.rcut2 = rcut2;
        desc[w] = d;
        order[w] = w;
    }
}

}  // namespace

extern "C" int pgf_force_device_noalloc(int n_walk, const int64_t* walk_table, const double* epi, int64_t n_epi_total,
                                        const pgf_epj_device* epj, const double* epj_r_search, int64_t n_epj_total,
                                        const pgf_spj_device* spj, int64_t n_spj_total, const int* id_epj,
                                        int64_t n_id_epj, const int* id_spj, int64_t n_id_spj, double eps2,
                                        double rcut2, double G, double* accp, int* n_ngb, void* cuda_stream,
                                        char* errbuf, size_t errbuf_len) {
    if (n_walk < 0 || n_walk > kMaxWalks)
        return fail(errbuf, errbuf_len, PGF_ERR_CAPACITY, "pgf_force_device_noalloc: %d walks; this entry point takes at most %d",
                    n_walk, kMaxWalks);
    if (n_epi_total < 0 || n_epj_total < 0 || n_spj_total < 0 || n_id_epj < 0 || n_id_spj < 0)
        return fail(errbuf, errbuf_len, PGF_ERR_ARG, "pgf_force_device_noalloc: negative array size");
    if (n_epi_total > 0x7fffffff || n_epj_total > 0x7fffffff || n_spj_total > 0x7fffffff)
        return fail(errbuf, errbuf_len, PGF_ERR_CAPACITY, "pgf_force_device_noalloc: more than 2^31-1 rows");
    if (!(eps2 >= 0) || !(rcut2 >= 0)) return fail(errbuf, errbuf_len, PGF_ERR_ARG, "pgf_force_device_noalloc: eps2, rcut2 < 0");
    if (n_walk == 0) return PGF_OK;
    if (!walk_table || (n_epi_total && (!epi || !accp || !n_ngb)) || (n_epj_total && (!epj || !epj_r_search)) ||
        (n_spj_total && !spj) || (n_id_epj && !id_epj) || (n_id_spj && !id_spj))
        return fail(errbuf, errbuf_len, PGF_ERR_ARG, "pgf_force_device_noalloc: NULL device array");
    if ((reinterpret_cast<uintptr_t>(accp) | reinterpret_cast<uintptr_t>(epj) | reinterpret_cast<uintptr_t>(spj) |
         reinterpret_cast<uintptr_t>(epi)) & 31)
        return fail(errbuf, errbuf_len, PGF_ERR_ARG, "pgf_force_device_noalloc: epi, epj, spj and accp must be 32-byte aligned");
    if ((reinterpret_cast<uintptr_t>(walk_table) | reinterpret_cast<uintptr_t>(epj_r_search)) & 7)
        return fail(errbuf, errbuf_len, PGF_ERR_ARG, "pgf_force_device_noalloc: walk_table and epj_r_search must be 8-byte aligned");
    if ((reinterpret_cast<uintptr_t>(id_epj) | reinterpret_cast<uintptr_t>(id_spj) | reinterpret_cast<uintptr_t>(n_ngb)) & 3)
        return fail(errbuf, errbuf_len, PGF_ERR_ARG, "pgf_force_device_noalloc: id_epj, id_spj and n_ngb must be 4-byte aligned");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(errbuf, errbuf_len, PGF_ERR_NO_DEVICE, "pgf_force_device_noalloc: %s", cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(errbuf, errbuf_len, PGF_ERR_NO_DEVICE, "pgf_force_device_noalloc: device %d", dev);
    cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
    if (s) {
        // The scratch address below belongs to the current device; work
        // queued on another device's stream would use that device's array
        // through the wrong address.
        int sdev = -1;
        e = cudaStreamGetDevice(s, &sdev);
        if (e != cudaSuccess) return fail(errbuf, errbuf_len, PGF_ERR_ARG, "pgf_force_device_noalloc: stream: %s", cudaGetErrorString(e));
        if (sdev != dev)
            return fail(errbuf, errbuf_len, PGF_ERR_ARG,
                        "pgf_force_device_noalloc: the stream belongs to device %d, the current device is %d", sdev, dev);
    }
    if (!g_scratch_addr[dev]) {
        unsigned char* ptr = nullptr;
        e = cudaGetSymbolAddress(reinterpret_cast<void**>(&ptr), g_noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            return fail(errbuf, errbuf_len, PGF_ERR_CUDA, "pgf_force_device_noalloc: scratch address: %s", cudaGetErrorString(e));
        int sms = 0;
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return fail(errbuf, errbuf_len, PGF_ERR_CUDA, "pgf_force_device_noalloc: %s", cudaGetErrorString(e));
        g_num_sms[dev] = sms;
        g_scratch_addr[dev] = ptr;
    }
    unsigned char* base = g_scratch_addr[dev];
    int32_t* flags = reinterpret_cast<int32_t*>(base + kFlagsOff);
    WalkDesc* desc = reinterpret_cast<WalkDesc*>(base + kDescOff);
    int32_t* order = reinterpret_cast<int32_t*>(base + kOrderOff);
    Retest* retest = reinterpret_cast<Retest*>(base + kRetestOff);

    e = cudaMemsetAsync(flags, 0, 3 * sizeof(int32_t), s);
    if (e != cudaSuccess) return fail(errbuf, errbuf_len, PGF_ERR_CUDA, "pgf_force_device_noalloc: %s", cudaGetErrorString(e));
    walk_prep_kernel<<<n_walk, 128, 0, s>>>(n_walk, walk_table, epi, n_epi_total, n_epj_total, n_spj_total, id_epj,
                                            n_id_epj, id_spj, n_id_spj, rcut2, desc, order, flags + 2);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(errbuf, errbuf_len, PGF_ERR_CUDA, "pgf_force_device_noalloc: prep: %s", cudaGetErrorString(e));
    // The interaction kernels trust the lists, so the validation result is
    // read back (into this stack variable) before they are launched.
    int32_t err_bits = 0;
    e = cudaMemcpyAsync(&err_bits, flags + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(errbuf, errbuf_len, PGF_ERR_CUDA, "pgf_force_device_noalloc: %s", cudaGetErrorString(e));
    if (err_bits)
        return fail(errbuf, errbuf_len, PGF_ERR_ARG, "pgf_force_device_noalloc: %s%s%s", (err_bits & kBadWalk) ? "walk table row out of range; " : "",
                    (err_bits & kBadEpjId) ? "EPJ id out of range; " : "", (err_bits & kBadSpjId) ? "SPJ id out of range" : "");

    Params p{};
    p.epi = reinterpret_cast<const EpiDev*>(epi);
    p.epj = reinterpret_cast<const EpjMix*>(epj);
    p.epj_m64 = nullptr;
    p.epj_rs64 = epj_r_search;
    p.spj = reinterpret_cast<const SpjMix*>(spj);
    p.spj_q64 = nullptr;
    p.id_epj = id_epj;
    p.id_spj = id_spj;
    p.walks = desc;
    p.order = order;
    p.n_walk = n_walk;
    p.eps2 = eps2;
    p.G = G;
    p.out_accp = reinterpret_cast<Accp*>(accp);
    p.out_nnb = n_ngb;
    p.queue_head = flags;
    p.n_retest = flags + 1;
    p.retest = retest;
    p.retest_cap = kRetestCap;
    p.err = flags + 2;
    e = launch_mixed(p, s, g_num_sms[dev]);
    if (e == cudaSuccess) e = launch_retest(p, s, g_num_sms[dev]);
    if (e != cudaSuccess) return fail(errbuf, errbuf_len, PGF_ERR_CUDA, "pgf_force_device_noalloc: launch: %s", cudaGetErrorString(e));
    return PGF_OK;
}
