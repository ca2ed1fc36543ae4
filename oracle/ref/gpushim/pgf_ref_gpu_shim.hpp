// Stand-ins for the FDPS / PeTar declarations that the reference's CUDA
// soft-force file (src/force_gpu_cuda.cu) expects from <particle_simulator.hpp>
// and "force_gpu_cuda.hpp", so that its device code compiles on its own into a
// cubin (oracle/ref/build_ref_gpu.sh).  Only the kernels
// force_kernel_ep_ep / force_kernel_ep_sp of that cubin are ever run; the host
// functor bodies are parsed but not compiled for the device.  Member names and
// meanings follow src/soft_ptcl.hpp:4-24 (ForceSoft), :271-308 (EPISoft),
// :311-376 (EPJSoft), FDPS's SPJQuadrupoleInAndOut (mass, pos, quad) and the
// functor declarations of src/force_gpu_cuda.hpp:101-168 (GPU_PROFILE form).
#pragma once
#include <cstdint>

namespace PS {
typedef int S32;
typedef long long S64;
typedef double F64;
typedef float F32;
struct F64vec {
    double x, y, z;
};
struct F64mat {
    double xx, yy, zz, xy, xz, yz;
};
}  // namespace PS

class ForceSoft {
public:
    PS::F64vec acc;
    PS::F64 pot;
    PS::S64 n_ngb;
};

class EPISoft {
public:
    PS::S64 id;
    PS::F64vec pos;
    PS::F64 r_search;
};

class EPJSoft {
public:
    PS::S64 id;
    PS::F64 mass;
    PS::F64vec pos;
    PS::F64 r_search;
};

class SPJQuadStandIn {
public:
    PS::F64 mass;
    PS::F64vec pos;
    PS::F64mat quad;
    PS::F64 getCharge() const { return mass; }
};
#define SPJSoft SPJQuadStandIn

// Profiling stand-ins (src/force_gpu_cuda.hpp:6-93): timers with start/end and
// an accumulated time, counters that add.
struct PgfRefTimer {
    double time = 0;
    void start() {}
    void end() {}
};
struct GPUProfile {
    PgfRefTimer copy, send, recv, calc;
};
struct GPUCounter {
    long long n_walk = 0, n_epi = 0, n_epj = 0, n_spj = 0, n_call = 0;
};
extern GPUProfile gpu_profile;
extern GPUCounter gpu_counter;

struct CalcForceWithLinearCutoffCUDAMultiWalk {
    PS::S32 my_rank;
    PS::F64 eps2;
    PS::F64 rcut2;
    PS::F64 G;
    PS::S32 operator()(const PS::S32 tag, const PS::S32 n_walk, const EPISoft** epi, const PS::S32* n_epi,
                       const PS::S32** id_epj, const PS::S32* n_epj, const PS::S32** id_spj, const PS::S32* n_spj,
                       const EPJSoft* epj, const PS::S32 n_epj_tot, const SPJSoft* spj, const PS::S32 n_spj_tot,
                       const bool send_flag);
};

PS::S32 RetrieveForceCUDA(const PS::S32 tag, const PS::S32 n_walk, const PS::S32* ni, ForceSoft** force);
