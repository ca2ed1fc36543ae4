// Header-only C++ functors with the signatures of PeTar's CUDA soft-force
// functors, implemented over the C ABI in petar_gpuforce.h.  Including this
// header instead of src/force_gpu_cuda.hpp lets src/petar.hpp:887-907 compile
// unchanged:
//   CalcForceWithLinearCutoffCUDAMultiWalk   src/force_gpu_cuda.hpp:103-133
//   CalcForceWithLinearCutoffCUDA            src/force_gpu_cuda.hpp:137-162
//   RetrieveForceCUDA                        src/force_gpu_cuda.hpp:165-168
//
// The including translation unit must define EPISoft, EPJSoft, ForceSoft and
// SPJSoft (PeTar: src/soft_ptcl.hpp and the SPJSoft macro of
// src/force_gpu_cuda.hpp:95-99) and the PS integer/float typedefs before
// including this file.  Field offsets are taken with offsetof, so the kernels
// read FDPS's arrays in place.  A non-zero status from the library aborts with
// its message, keeping the reference's assert-on-failure behaviour
// (src/force_gpu_cuda.cu:548,634-636).
#pragma once
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "petar_gpuforce.h"

namespace petar_gpuforce {

inline void check(int code, const char* what) {
    if (code != PGF_OK) {
        std::fprintf(stderr, "petar_gpuforce: %s failed (%d): %s\n", what, code, pgf_last_error());
        std::abort();
    }
}

template <class Tepi>
inline pgf_epi_layout epi_layout() {
    return pgf_epi_layout{sizeof(Tepi), offsetof(Tepi, pos), offsetof(Tepi, r_search)};
}

template <class Tepj>
inline pgf_epj_layout epj_layout() {
    return pgf_epj_layout{sizeof(Tepj), offsetof(Tepj, mass), offsetof(Tepj, pos), offsetof(Tepj, r_search)};
}

// Superparticles with a quadrupole member (FDPS SPJQuadrupole*) or without
// one (SPJMonopole*).
template <class T, class = void>
struct has_quad : std::false_type {};
template <class T>
struct has_quad<T, decltype((void)offsetof(T, quad))> : std::true_type {};

template <class Tspj>
inline pgf_spj_layout spj_layout() {
    pgf_spj_layout l{sizeof(Tspj), offsetof(Tspj, mass), offsetof(Tspj, pos), 0, 0};
    if constexpr (has_quad<Tspj>::value) {
        l.off_quad = offsetof(Tspj, quad);
        l.has_quad = 1;
    }
    return l;
}

template <class Tforce>
inline pgf_force_layout force_layout() {
    return pgf_force_layout{sizeof(Tforce), offsetof(Tforce, acc), offsetof(Tforce, pot), offsetof(Tforce, n_ngb),
                            (int)sizeof(((Tforce*)nullptr)->n_ngb)};
}

}  // namespace petar_gpuforce

struct CalcForceWithLinearCutoffCUDAMultiWalk {
    PS::S32 my_rank;
    PS::F64 eps2;
    PS::F64 rcut2;
    PS::F64 G;

    CalcForceWithLinearCutoffCUDAMultiWalk() {}
    CalcForceWithLinearCutoffCUDAMultiWalk(PS::S32 _rank, PS::F64 _eps2, PS::F64 _rcut2, PS::F64 _G)
        : my_rank(_rank), eps2(_eps2), rcut2(_rcut2), G(_G) {}

    void initialize(PS::S32 _rank, PS::F64 _eps2, PS::F64 _rcut2, PS::F64 _G) {
        my_rank = _rank;
        eps2 = _eps2;
        rcut2 = _rcut2;
        G = _G;
    }

    PS::S32 operator()(const PS::S32 tag, const PS::S32 n_walk, const EPISoft** epi, const PS::S32* n_epi,
                       const PS::S32** id_epj, const PS::S32* n_epj, const PS::S32** id_spj, const PS::S32* n_spj,
                       const EPJSoft* epj, const PS::S32 n_epj_tot, const SPJSoft* spj, const PS::S32 n_spj_tot,
                       const bool send_flag) {
        using namespace petar_gpuforce;
        check(pgf_initialize(my_rank, eps2, rcut2, G), "pgf_initialize");
        check(pgf_set_mode(PGF_MODE_FORCE), "pgf_set_mode");
        const pgf_epi_layout il = epi_layout<EPISoft>();
        const pgf_epj_layout jl = epj_layout<EPJSoft>();
        const pgf_spj_layout sl = spj_layout<SPJSoft>();
        check(pgf_dispatch_index(tag, n_walk, reinterpret_cast<const void* const*>(epi), n_epi, &il,
                                 reinterpret_cast<const int* const*>(id_epj), n_epj,
                                 reinterpret_cast<const int* const*>(id_spj), n_spj, epj, n_epj_tot, &jl, spj,
                                 n_spj_tot, &sl, send_flag ? 1 : 0),
              "pgf_dispatch_index");
        return 0;
    }
};

struct CalcForceWithLinearCutoffCUDA {
    PS::S32 my_rank;
    PS::F64 eps2;
    PS::F64 rcut2;
    PS::F64 G;

    CalcForceWithLinearCutoffCUDA() {}
    CalcForceWithLinearCutoffCUDA(PS::S32 _rank, PS::F64 _eps2, PS::F64 _rcut2, PS::F64 _G)
        : my_rank(_rank), eps2(_eps2), rcut2(_rcut2), G(_G) {}

    void initialize(PS::S32 _rank, PS::F64 _eps2, PS::F64 _rcut2, PS::F64 _G) {
        my_rank = _rank;
        eps2 = _eps2;
        rcut2 = _rcut2;
        G = _G;
    }

    PS::S32 operator()(const PS::S32 tag, const PS::S32 n_walk, const EPISoft* epi[], const PS::S32 n_epi[],
                       const EPJSoft* epj[], const PS::S32 n_epj[], const SPJSoft* spj[], const PS::S32 n_spj[]) {
        using namespace petar_gpuforce;
        check(pgf_initialize(my_rank, eps2, rcut2, G), "pgf_initialize");
        check(pgf_set_mode(PGF_MODE_FORCE), "pgf_set_mode");
        const pgf_epi_layout il = epi_layout<EPISoft>();
        const pgf_epj_layout jl = epj_layout<EPJSoft>();
        const pgf_spj_layout sl = spj_layout<SPJSoft>();
        check(pgf_dispatch(tag, n_walk, reinterpret_cast<const void* const*>(epi), n_epi, &il,
                           reinterpret_cast<const void* const*>(epj), n_epj, &jl,
                           reinterpret_cast<const void* const*>(spj), n_spj, &sl),
              "pgf_dispatch");
        return 0;
    }
};

// Multi-walk GPU form of SearchNeighborEpEpNoSimd (src/soft_force.hpp:11-34):
// the same dispatch signature as the force functor; RetrieveForceCUDA then
// overwrites n_ngb only.  Counts use r^2 < max(rs_i, rs_j)^2 without
// softening; SPJ lists are ignored.
struct SearchNeighborEpEpCUDAMultiWalk {
    PS::S32 my_rank;
    PS::F64 eps2;
    PS::F64 rcut2;
    PS::F64 G;

    SearchNeighborEpEpCUDAMultiWalk() {}
    SearchNeighborEpEpCUDAMultiWalk(PS::S32 _rank, PS::F64 _eps2, PS::F64 _rcut2, PS::F64 _G)
        : my_rank(_rank), eps2(_eps2), rcut2(_rcut2), G(_G) {}

    PS::S32 operator()(const PS::S32 tag, const PS::S32 n_walk, const EPISoft** epi, const PS::S32* n_epi,
                       const PS::S32** id_epj, const PS::S32* n_epj, const PS::S32** id_spj, const PS::S32* n_spj,
                       const EPJSoft* epj, const PS::S32 n_epj_tot, const SPJSoft* spj, const PS::S32 n_spj_tot,
                       const bool send_flag) {
        using namespace petar_gpuforce;
        check(pgf_initialize(my_rank, eps2, rcut2, G), "pgf_initialize");
        check(pgf_set_mode(PGF_MODE_NEIGHBOR_SEARCH), "pgf_set_mode");
        const pgf_epi_layout il = epi_layout<EPISoft>();
        const pgf_epj_layout jl = epj_layout<EPJSoft>();
        const pgf_spj_layout sl = spj_layout<SPJSoft>();
        check(pgf_dispatch_index(tag, n_walk, reinterpret_cast<const void* const*>(epi), n_epi, &il,
                                 reinterpret_cast<const int* const*>(id_epj), n_epj,
                                 reinterpret_cast<const int* const*>(id_spj), n_spj, epj, n_epj_tot, &jl, spj,
                                 n_spj_tot, &sl, send_flag ? 1 : 0),
              "pgf_dispatch_index");
        return 0;
    }
};

inline PS::S32 RetrieveForceCUDA(const PS::S32 tag, const PS::S32 n_walk, const PS::S32* ni, ForceSoft** force) {
    using namespace petar_gpuforce;
    const pgf_force_layout fl = force_layout<ForceSoft>();
    check(pgf_retrieve(tag, n_walk, ni, reinterpret_cast<void* const*>(force), &fl), "pgf_retrieve");
    return 0;
}

// ---- Fused changeover mode (no counterpart in the reference, whose
// correction runs on the CPU after the kernel, src/hard.hpp:1656-1693) ----
//
// Tepi is PeTar's EPISoft extended with the particle's changeover radii and
// the mass of its self-potential term (members: fields id, pos, r_search,
// r_in, r_out, self_mass); Tforce is ForceSoft extended with pot_soft.  The
// EPJ side uses EPJSoft's own id, r_in, r_out and group_data, whose
// artificial-particle information starts with (mass_backup, status)
// (src/artificial_particles.hpp:20-23).  After retrieve, pot holds pot_tot
// and pot_soft the soft potential; FPSoft takes them instead of copying pot
// into both (src/soft_ptcl.hpp:84-95), and the CPU correction pass is skipped.
namespace petar_gpuforce {
template <class Tepi, class Tepj, class Tforce>
inline pgf_changeover_layout changeover_layout() {
    pgf_changeover_layout l;
    l.epi_off_id = offsetof(Tepi, id);
    l.epi_off_r_in = offsetof(Tepi, r_in);
    l.epi_off_r_out = offsetof(Tepi, r_out);
    l.epi_off_self_mass = offsetof(Tepi, self_mass);
    l.epj_off_id = offsetof(Tepj, id);
    l.epj_off_r_in = offsetof(Tepj, r_in);
    l.epj_off_r_out = offsetof(Tepj, r_out);
    l.epj_off_mass_backup = offsetof(Tepj, group_data);
    l.epj_off_status = offsetof(Tepj, group_data) + sizeof(double);
    l.force_off_pot_soft = offsetof(Tforce, pot_soft);
    return l;
}
}  // namespace petar_gpuforce

template <class Tepi, class Tforce>
struct CalcForceWithLinearCutoffChangeoverCUDAMultiWalk {
    PS::S32 my_rank;
    PS::F64 eps2;
    PS::F64 rcut2;
    PS::F64 G;

    CalcForceWithLinearCutoffChangeoverCUDAMultiWalk() {}
    CalcForceWithLinearCutoffChangeoverCUDAMultiWalk(PS::S32 _rank, PS::F64 _eps2, PS::F64 _rcut2, PS::F64 _G)
        : my_rank(_rank), eps2(_eps2), rcut2(_rcut2), G(_G) {}

    PS::S32 operator()(const PS::S32 tag, const PS::S32 n_walk, const Tepi** epi, const PS::S32* n_epi,
                       const PS::S32** id_epj, const PS::S32* n_epj, const PS::S32** id_spj, const PS::S32* n_spj,
                       const EPJSoft* epj, const PS::S32 n_epj_tot, const SPJSoft* spj, const PS::S32 n_spj_tot,
                       const bool send_flag) {
        using namespace petar_gpuforce;
        check(pgf_initialize(my_rank, eps2, rcut2, G), "pgf_initialize");
        const pgf_changeover_layout col = changeover_layout<Tepi, EPJSoft, Tforce>();
        check(pgf_set_changeover_layout(&col), "pgf_set_changeover_layout");
        check(pgf_set_mode(PGF_MODE_FORCE_CHANGEOVER), "pgf_set_mode");
        const pgf_epi_layout il = epi_layout<Tepi>();
        const pgf_epj_layout jl = epj_layout<EPJSoft>();
        const pgf_spj_layout sl = spj_layout<SPJSoft>();
        check(pgf_dispatch_index(tag, n_walk, reinterpret_cast<const void* const*>(epi), n_epi, &il,
                                 reinterpret_cast<const int* const*>(id_epj), n_epj,
                                 reinterpret_cast<const int* const*>(id_spj), n_spj, epj, n_epj_tot, &jl, spj,
                                 n_spj_tot, &sl, send_flag ? 1 : 0),
              "pgf_dispatch_index");
        return 0;
    }
};

template <class Tforce>
inline PS::S32 RetrieveForceChangeoverCUDA(const PS::S32 tag, const PS::S32 n_walk, const PS::S32* ni,
                                           Tforce** force) {
    using namespace petar_gpuforce;
    const pgf_force_layout fl = force_layout<Tforce>();
    check(pgf_retrieve(tag, n_walk, ni, reinterpret_cast<void* const*>(force), &fl), "pgf_retrieve");
    return 0;
}
