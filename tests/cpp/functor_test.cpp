// Drives the header-only functors (include/petar_gpuforce.hpp) the way FDPS
// and the reference kernel test do (src/simd_test.cxx:142-155): one
// send_flag=true call with the shared EPJ/SPJ arrays, one send_flag=false call
// with per-walk EPI pointers and id lists, then RetrieveForceCUDA into
// per-walk ForceSoft arrays.  The record types below have the field order of
// PeTar's EPISoft / EPJSoft / ForceSoft (src/soft_ptcl.hpp) and of FDPS's
// quadrupole superparticle; no FDPS headers are needed.
//
// Input (binary, little endian): int64 n_walk, n_epj, n_spj, n_i_tot, n_idj,
// n_ids; double eps2, rcut2, G; int32 n_epi[n_walk], n_epj[n_walk],
// n_spj[n_walk]; double epi_pos[3 n_i_tot], epi_rs[n_i_tot], epj_mass[n_epj],
// epj_pos[3 n_epj], epj_rs[n_epj], spj_mass[n_spj], spj_pos[3 n_spj],
// spj_quad[6 n_spj]; int32 id_epj[n_idj], id_spj[n_ids].
// Output: double acc[3 n_i_tot], pot[n_i_tot]; int64 n_ngb[n_i_tot].
#include <cstdint>
#include <cstdio>
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

struct SPJQuadrupoleTest {
    PS::F64 mass;
    PS::F64vec pos;
    PS::F64mat quad;
};
#define SPJSoft SPJQuadrupoleTest

struct ForceSoft {
    PS::F64vec acc;
    PS::F64 pot;
    PS::S64 n_ngb;
};

#include "petar_gpuforce.hpp"

// Records of the fused changeover mode: EPISoft and ForceSoft extended.
struct EPISoftCO {
    PS::S64 id;
    PS::F64vec pos;
    PS::F64 r_search;
    PS::S32 rank_org;
    PS::S32 type;
    PS::F64 r_in, r_out, self_mass;
};
struct ForceSoftCO {
    PS::F64vec acc;
    PS::F64 pot;
    PS::S64 n_ngb;
    PS::F64 pot_soft;
};
// The changeover functor and retrieve instantiate with them (compile check).
template struct CalcForceWithLinearCutoffChangeoverCUDAMultiWalk<EPISoftCO, ForceSoftCO>;
template PS::S32 RetrieveForceChangeoverCUDA<ForceSoftCO>(const PS::S32, const PS::S32, const PS::S32*, ForceSoftCO**);

template <class T>
static void rd(FILE* f, T* p, size_t n) {
    if (n && fread(p, sizeof(T), n, f) != n) {
        std::fprintf(stderr, "short read\n");
        std::exit(2);
    }
}

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int64_t h[6];
    double par[3];
    rd(f, h, 6);
    rd(f, par, 3);
    const int64_t nw = h[0], nej = h[1], nsj = h[2], ni = h[3], nidj = h[4], nids = h[5];
    std::vector<int32_t> n_epi(nw), n_epj(nw), n_spj(nw);
    rd(f, n_epi.data(), nw);
    rd(f, n_epj.data(), nw);
    rd(f, n_spj.data(), nw);
    std::vector<double> epi_pos(3 * ni), epi_rs(ni), epj_mass(nej), epj_pos(3 * nej), epj_rs(nej), spj_mass(nsj),
        spj_pos(3 * nsj), spj_quad(6 * nsj);
    rd(f, epi_pos.data(), 3 * ni);
    rd(f, epi_rs.data(), ni);
    rd(f, epj_mass.data(), nej);
    rd(f, epj_pos.data(), 3 * nej);
    rd(f, epj_rs.data(), nej);
    rd(f, spj_mass.data(), nsj);
    rd(f, spj_pos.data(), 3 * nsj);
    rd(f, spj_quad.data(), 6 * nsj);
    std::vector<int32_t> id_epj(nidj), id_spj(nids);
    rd(f, id_epj.data(), nidj);
    rd(f, id_spj.data(), nids);
    std::fclose(f);

    std::vector<EPISoft> epi(ni);
    for (int64_t i = 0; i < ni; ++i) {
        epi[i] = EPISoft{i, {epi_pos[3 * i], epi_pos[3 * i + 1], epi_pos[3 * i + 2]}, epi_rs[i], 0, 1};
    }
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
        idj_ptr[w] = id_epj.data() + oj;
        ids_ptr[w] = id_spj.data() + os;
        oi += n_epi[w];
        oj += n_epj[w];
        os += n_spj[w];
    }
    CalcForceWithLinearCutoffCUDAMultiWalk calc(0, par[0], par[1], par[2]);
    calc(1, 0, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, epj.data(), (PS::S32)nej, spj.data(),
      (PS::S32)nsj, true);
    calc(1, (PS::S32)nw, epi_ptr.data(), n_epi.data(), idj_ptr.data(), n_epj.data(), ids_ptr.data(), n_spj.data(),
      epj.data(), (PS::S32)nej, spj.data(), (PS::S32)nsj, false);
    RetrieveForceCUDA(1, (PS::S32)nw, n_epi.data(), force_ptr.data());

    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 2;
    for (int64_t i = 0; i < ni; ++i) std::fwrite(&force[i].acc, sizeof(double), 3, o);
    for (int64_t i = 0; i < ni; ++i) std::fwrite(&force[i].pot, sizeof(double), 1, o);
    for (int64_t i = 0; i < ni; ++i) std::fwrite(&force[i].n_ngb, sizeof(int64_t), 1, o);
    std::fclose(o);
    pgf_finalize();
    return 0;
}
