// PeTar's unchanged call pattern timed from C++: the header-only functors of
// include/petar_gpuforce.hpp with PeTar-layout records, driven the way FDPS's
// multi-walk loop calls them with PeTar's settings (src/petar.hpp:888-899:
// one tag, n_walk_limit walks per call): one send_flag=true call with the
// shared EPJ/SPJ arrays, then per batch of walks one send_flag=false call and
// one RetrieveForceCUDA.  The record types have the field order of PeTar's
// EPISoft / EPJSoft / ForceSoft (src/soft_ptcl.hpp) and of FDPS's quadrupole
// superparticle; no FDPS headers are needed.  Loaded by bench.py (ctypes).
#include <chrono>
#include <cstdint>
#include <vector>

namespace PS {
typedef int S32;
typedef long long S64;
typedef double F64;
struct F64vec {
    double x, y, z;
};
struct F64mat {
    double xx, yy, zz, xy, xz, yz;
};
}  // namespace PS

struct EPISoft {
    PS::S64 id;
    PS::F64vec pos;
    PS::F64 r_search;
    PS::S32 rank_org;
    PS::S32 type;
};

struct EPJSoft {
    PS::S64 id;
    PS::F64 mass;
    PS::F64vec pos;
    PS::F64vec vel;
    PS::F64 r_in, r_out, r_search, r_scale_next;
    PS::S64 group_data[2];
    PS::S32 rank_org, adr_org;
};

struct SPJQuadrupoleBench {
    PS::F64 mass;
    PS::F64vec pos;
    PS::F64mat quad;
};
#define SPJSoft SPJQuadrupoleBench

struct ForceSoft {
    PS::F64vec acc;
    PS::F64 pot;
    PS::S64 n_ngb;
};

#include "petar_gpuforce.hpp"

// Builds the records once, then runs `reps` force evaluations of all n_walk
// walks in calls of `batch` walks and returns the fastest evaluation's time in
// *ms.  acc (3 per i), pot and nnb, when given, receive the last results.
extern "C" int fdps_batches_run(int64_t nw, const int32_t* n_epi, const int32_t* n_epj, const int32_t* n_spj,
                                const double* epi_pos, const double* epi_rs, int64_t nej, const double* epj_mass,
                                const double* epj_pos, const double* epj_rs, int64_t nsj, const double* spj_mass,
                                const double* spj_pos, const double* spj_quad, const int32_t* id_epj,
                                const int32_t* id_spj, double eps2, double rcut2, double G, int batch, int reps,
                                double* ms, double* acc, double* pot, int64_t* nnb) {
    if (nw <= 0 || batch <= 0 || reps <= 0) return 1;
    int64_t ni = 0, nidj = 0, nids = 0;
    for (int64_t w = 0; w < nw; ++w) {
        ni += n_epi[w];
        nidj += n_epj[w];
        nids += n_spj[w];
    }
    std::vector<EPISoft> epi(ni);
    for (int64_t i = 0; i < ni; ++i)
        epi[i] = EPISoft{i, {epi_pos[3 * i], epi_pos[3 * i + 1], epi_pos[3 * i + 2]}, epi_rs[i], 0, 1};
    std::vector<EPJSoft> epj(nej);
    for (int64_t j = 0; j < nej; ++j) {
        EPJSoft e{};
        e.id = j;
        e.mass = epj_mass[j];
        e.pos = {epj_pos[3 * j], epj_pos[3 * j + 1], epj_pos[3 * j + 2]};
        e.r_search = epj_rs[j];
        epj[j] = e;
    }
    std::vector<SPJSoft> spj(nsj);
    for (int64_t j = 0; j < nsj; ++j) {
        const double* q = &spj_quad[6 * j];
        spj[j] = SPJSoft{spj_mass[j], {spj_pos[3 * j], spj_pos[3 * j + 1], spj_pos[3 * j + 2]},
                         {q[0], q[1], q[2], q[3], q[4], q[5]}};
    }
    std::vector<const EPISoft*> epi_ptr(nw);
    std::vector<const PS::S32*> idj_ptr(nw), ids_ptr(nw);
    std::vector<ForceSoft> force(ni);
    std::vector<ForceSoft*> force_ptr(nw);
    int64_t oi = 0, oj = 0, os = 0;
    for (int64_t w = 0; w < nw; ++w) {
        epi_ptr[w] = epi.data() + oi;
        force_ptr[w] = force.data() + oi;
        idj_ptr[w] = id_epj + oj;
        ids_ptr[w] = id_spj + os;
        oi += n_epi[w];
        oj += n_epj[w];
        os += n_spj[w];
    }
    CalcForceWithLinearCutoffCUDAMultiWalk calc(0, eps2, rcut2, G);
    double best = 1e300;
    for (int r = 0; r <= reps; ++r) {  // the first evaluation warms up
        const auto t0 = std::chrono::steady_clock::now();
        calc(0, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, epj.data(), (PS::S32)nej, spj.data(),
             (PS::S32)nsj, true);
        for (int64_t w0 = 0; w0 < nw; w0 += batch) {
            const int n = (int)(nw - w0 < batch ? nw - w0 : batch);
            calc(0, n, epi_ptr.data() + w0, n_epi + w0, idj_ptr.data() + w0, n_epj + w0, ids_ptr.data() + w0,
                 n_spj + w0, epj.data(), (PS::S32)nej, spj.data(), (PS::S32)nsj, false);
            RetrieveForceCUDA(0, n, n_epi + w0, force_ptr.data() + w0);
        }
        const double t = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (r > 0 && t < best) best = t;
    }
    *ms = best;
    for (int64_t i = 0; i < ni; ++i) {
        if (acc) {
            acc[3 * i] = force[i].acc.x;
            acc[3 * i + 1] = force[i].acc.y;
            acc[3 * i + 2] = force[i].acc.z;
        }
        if (pot) pot[i] = force[i].pot;
        if (nnb) nnb[i] = force[i].n_ngb;
    }
    return 0;
}
