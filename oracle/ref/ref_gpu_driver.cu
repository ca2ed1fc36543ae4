// Runs the reference's own CUDA soft-force kernels (force_kernel_ep_ep and
// force_kernel_ep_sp of src/force_gpu_cuda.cu, compiled from the reference
// sources into oracle/_ref/ref_force_gpu.cubin by build_ref_gpu.sh) on a
// multi-walk batch, for comparison with the oracle and the library's kernels.
// Test infrastructure only.
//
// The host side restates what the reference functor does before and after the
// launches (src/force_gpu_cuda.cu:621-699 and 831-880): positions, masses,
// r_search and quadrupoles rounded to FP32 into the kernels' record layouts,
// EPI rows tagged with their walk, ij_disp prefix sums with a repeated last
// row, the EPI rows padded to a multiple of 32 with walk index n_walk, one
// 32-thread block per 32 rows, the EP-EP kernel then the EP-SP kernel, and
// the FP32 results widened to FP64.
//
// Bounds.  The kernels gather epj[id_epj[j + tid]] for all 32 lanes of the
// last tile of a list, up to 31 entries past its end
// (src/force_gpu_cuda.cu:100,154-155,173; SPJ at :345,398-399,417), and read
// ij_disp[n_walk + 1].  So every id is checked on the host, both id arrays
// carry 32 zero entries after the last list (id 0 is a valid row: each j
// array holds at least one record, zeroed when the batch has none), ij_disp
// has n_walk + 2 rows, and padding rows are zeroed.  Every gather then stays
// inside its allocation.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace {

// Record layouts of src/force_gpu_cuda.cu:19-47 (USE_QUAD).
struct EpiGPU {
    float3 pos;
    float r_search;
    int id_walk;
};
struct EpjGPU {
    float3 pos;
    float m;
    float r_search;
};
struct SpjGPU {
    float3 pos;
    float m;
    float qxx, qyy, qzz, qxy, qxz, qyz;
};
struct ForceGPU {
    float4 accp;
    int nnb;
};
static_assert(sizeof(EpiGPU) == 20 && sizeof(EpjGPU) == 20 && sizeof(SpjGPU) == 40 && sizeof(ForceGPU) == 32,
              "reference record layouts");

constexpr int kThreads = 32;  // N_THREAD_GPU
constexpr int kPad = 32;      // zero ids after the last list

CUmodule g_mod = nullptr;
CUfunction g_epep = nullptr, g_epsp = nullptr;

int fail(char* err, size_t len, int code, const char* msg, const char* detail = "") {
    if (err && len) snprintf(err, len, "%s%s", msg, detail);
    return code;
}

template <class T>
struct Dev {
    T* p = nullptr;
    ~Dev() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, (n ? n : 1) * sizeof(T)); }
};

}  // namespace

extern "C" int ref_gpu_load(const char* cubin, char* err, size_t errlen) {
    if (g_mod) return 0;
    cudaError_t ce = cudaFree(nullptr);  // the runtime's primary context becomes current
    if (ce != cudaSuccess) return fail(err, errlen, 2, "no CUDA device: ", cudaGetErrorString(ce));
    CUresult r = cuModuleLoad(&g_mod, cubin);
    if (r != CUDA_SUCCESS) {
        g_mod = nullptr;
        return fail(err, errlen, 3, "cuModuleLoad failed for ", cubin);
    }
    // force_kernel_ep_ep(const int3*, const EpiGPU*, const EpjGPU*, const int*, ForceGPU*, float, float, float)
    // force_kernel_ep_sp(const int3*, const EpiGPU*, const SpjGPU*, const int*, ForceGPU*, float, float)
    if (cuModuleGetFunction(&g_epep, g_mod, "_Z18force_kernel_ep_epPK4int3PK6EpiGPUPK6EpjGPUPKiP8ForceGPUfff") !=
            CUDA_SUCCESS ||
        cuModuleGetFunction(&g_epsp, g_mod, "_Z18force_kernel_ep_spPK4int3PK6EpiGPUPK6SpjGPUPKiP8ForceGPUff") !=
            CUDA_SUCCESS) {
        cuModuleUnload(g_mod);
        g_mod = nullptr;
        return fail(err, errlen, 3, "kernels not found in ", cubin);
    }
    return 0;
}

// One evaluation of all n_walk walks (plus `repeats` timed re-runs of the two
// kernels; *ms_out receives their mean time).  Arrays follow the multi-walk
// batch layout: per-walk displacements into the EPI rows and the id lists.
extern "C" int ref_gpu_force(int n_walk, const int64_t* epi_disp, const double* epi_pos, const double* epi_rs,
                             const int64_t* epj_disp, const int32_t* id_epj, const int64_t* spj_disp,
                             const int32_t* id_spj, int64_t n_epj_tot, const double* epj_pos, const double* epj_mass,
                             const double* epj_rs, int64_t n_spj_tot, const double* spj_pos, const double* spj_mass,
                             const double* spj_quad, double eps2, double rcut2, double G, int repeats, double* acc,
                             double* pot, int64_t* nnb, double* ms_out, char* err, size_t errlen) {
    if (!g_mod) return fail(err, errlen, 4, "ref_gpu_load has not succeeded");
    if (n_walk <= 0) return 0;
    const int64_t ni = epi_disp[n_walk], ne = epj_disp[n_walk], ns = spj_disp[n_walk];
    if (ni <= 0) return 0;
    if (ni > INT32_MAX - kThreads || ne > INT32_MAX - kPad || ns > INT32_MAX - kPad || n_epj_tot > INT32_MAX ||
        n_spj_tot > INT32_MAX)
        return fail(err, errlen, 1, "sizes exceed the reference's int indexing");
    for (int w = 0; w < n_walk; ++w)
        if (epi_disp[w + 1] < epi_disp[w] || epj_disp[w + 1] < epj_disp[w] || spj_disp[w + 1] < spj_disp[w] ||
            epj_disp[0] != 0 || spj_disp[0] != 0 || epi_disp[0] != 0)
            return fail(err, errlen, 1, "displacements are not non-decreasing from 0");
    for (int64_t k = 0; k < ne; ++k)
        if (id_epj[k] < 0 || id_epj[k] >= n_epj_tot) return fail(err, errlen, 1, "EPJ id out of range");
    for (int64_t k = 0; k < ns; ++k)
        if (id_spj[k] < 0 || id_spj[k] >= n_spj_tot) return fail(err, errlen, 1, "SPJ id out of range");

    const int64_t ni_reg = (ni + kThreads - 1) / kThreads * kThreads;
    std::vector<int3> disp(n_walk + 2);
    disp[0] = make_int3(0, 0, 0);
    for (int w = 0; w < n_walk; ++w)
        disp[w + 1] = make_int3((int)epi_disp[w + 1], (int)epj_disp[w + 1], (int)spj_disp[w + 1]);
    disp[n_walk + 1] = disp[n_walk];
    std::vector<EpiGPU> hepi(ni_reg);
    std::memset(hepi.data(), 0, ni_reg * sizeof(EpiGPU));
    for (int w = 0; w < n_walk; ++w)
        for (int64_t i = epi_disp[w]; i < epi_disp[w + 1]; ++i)
            hepi[i] = EpiGPU{make_float3((float)epi_pos[3 * i], (float)epi_pos[3 * i + 1], (float)epi_pos[3 * i + 2]),
                             (float)epi_rs[i], w};
    for (int64_t i = ni; i < ni_reg; ++i) hepi[i].id_walk = n_walk;
    std::vector<EpjGPU> hepj(n_epj_tot > 0 ? n_epj_tot : 1);
    std::memset(hepj.data(), 0, hepj.size() * sizeof(EpjGPU));
    for (int64_t j = 0; j < n_epj_tot; ++j)
        hepj[j] = EpjGPU{make_float3((float)epj_pos[3 * j], (float)epj_pos[3 * j + 1], (float)epj_pos[3 * j + 2]),
                         (float)epj_mass[j], (float)epj_rs[j]};
    std::vector<SpjGPU> hspj(n_spj_tot > 0 ? n_spj_tot : 1);
    std::memset(hspj.data(), 0, hspj.size() * sizeof(SpjGPU));
    for (int64_t j = 0; j < n_spj_tot; ++j) {
        const double* q = spj_quad + 6 * j;
        hspj[j] = SpjGPU{make_float3((float)spj_pos[3 * j], (float)spj_pos[3 * j + 1], (float)spj_pos[3 * j + 2]),
                         (float)spj_mass[j], (float)q[0], (float)q[1], (float)q[2], (float)q[3], (float)q[4],
                         (float)q[5]};
    }
    std::vector<int32_t> he(ne + kPad, 0), hs(ns + kPad, 0);
    std::memcpy(he.data(), id_epj, ne * sizeof(int32_t));
    std::memcpy(hs.data(), id_spj, ns * sizeof(int32_t));

    Dev<int3> d_disp;
    Dev<EpiGPU> d_epi;
    Dev<EpjGPU> d_epj;
    Dev<SpjGPU> d_spj;
    Dev<int32_t> d_ide, d_ids;
    Dev<ForceGPU> d_force;
    cudaError_t e = cudaSuccess;
    if ((e = d_disp.alloc(disp.size())) || (e = d_epi.alloc(hepi.size())) || (e = d_epj.alloc(hepj.size())) ||
        (e = d_spj.alloc(hspj.size())) || (e = d_ide.alloc(he.size())) || (e = d_ids.alloc(hs.size())) ||
        (e = d_force.alloc(ni_reg)))
        return fail(err, errlen, 5, "cudaMalloc: ", cudaGetErrorString(e));
    if ((e = cudaMemcpy(d_disp.p, disp.data(), disp.size() * sizeof(int3), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(d_epi.p, hepi.data(), hepi.size() * sizeof(EpiGPU), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(d_epj.p, hepj.data(), hepj.size() * sizeof(EpjGPU), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(d_spj.p, hspj.data(), hspj.size() * sizeof(SpjGPU), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(d_ide.p, he.data(), he.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) ||
        (e = cudaMemcpy(d_ids.p, hs.data(), hs.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) ||
        (e = cudaMemset(d_force.p, 0, ni_reg * sizeof(ForceGPU))))
        return fail(err, errlen, 5, "copy: ", cudaGetErrorString(e));

    float feps2 = (float)eps2, frcut2 = (float)rcut2, fG = (float)G;
    void* a_ep[] = {&d_disp.p, &d_epi.p, &d_epj.p, &d_ide.p, &d_force.p, &feps2, &frcut2, &fG};
    void* a_sp[] = {&d_disp.p, &d_epi.p, &d_spj.p, &d_ids.p, &d_force.p, &feps2, &fG};
    const unsigned nblocks = (unsigned)(ni_reg / kThreads);
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float ms_sum = 0.f;
    for (int rep = 0; rep <= repeats; ++rep) {
        cudaEventRecord(t0, 0);
        CUresult r = cuLaunchKernel(g_epep, nblocks, 1, 1, kThreads, 1, 1, 0, 0, a_ep, nullptr);
        if (r == CUDA_SUCCESS) r = cuLaunchKernel(g_epsp, nblocks, 1, 1, kThreads, 1, 1, 0, 0, a_sp, nullptr);
        cudaEventRecord(t1, 0);
        if (r != CUDA_SUCCESS) {
            cudaEventDestroy(t0);
            cudaEventDestroy(t1);
            return fail(err, errlen, 6, "cuLaunchKernel failed");
        }
        if ((e = cudaEventSynchronize(t1)) != cudaSuccess) {
            cudaEventDestroy(t0);
            cudaEventDestroy(t1);
            return fail(err, errlen, 6, "kernels: ", cudaGetErrorString(e));
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t0, t1);
        if (rep > 0) ms_sum += ms;
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (ms_out) *ms_out = repeats > 0 ? ms_sum / repeats : 0.0;
    std::vector<ForceGPU> hf(ni);
    if ((e = cudaMemcpy(hf.data(), d_force.p, ni * sizeof(ForceGPU), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return fail(err, errlen, 5, "copy back: ", cudaGetErrorString(e));
    for (int64_t i = 0; i < ni; ++i) {
        acc[3 * i] = hf[i].accp.x;
        acc[3 * i + 1] = hf[i].accp.y;
        acc[3 * i + 2] = hf[i].accp.z;
        pot[i] = hf[i].accp.w;
        nnb[i] = hf[i].nnb;
    }
    return 0;
}
