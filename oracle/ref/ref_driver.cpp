// C entry points around the reference's own force functors, for building
// golden fixtures.  Compiled once per variant by build_ref.sh:
//   REF_NOSIMD : CalcForceEpEpWithLinearCutoffNoSimd, CalcForceEpSpQuadNoSimd,
//                SearchNeighborEpEpNoSimd  (src/soft_force.hpp:11-34,38-87,160-200)
//   REF_SIMD   : CalcForceEpEpWithLinearCutoffSimd, CalcForceEpSpQuadSimd,
//                SearchNeighborEpEpSimd    (src/soft_force.hpp:239-283,350-425,491-554)
//                over PhantomGrapeQuad (FP32) or, with CALC_EP_64bit /
//                CALC_SP_64bit, PhantomGrapeQuad64Bit.
// Each call evaluates one i-set against one j-set, as one FDPS walk would.
#include <vector>

#include "ref_shim.hpp"
#include "soft_force.hpp"

PS::F64 ForceSoft::grav_const = 1.0;
PS::F64 EPISoft::eps = 0.0;
PS::F64 EPISoft::r_out = 0.0;

#if defined(REF_NOSIMD)
typedef CalcForceEpEpWithLinearCutoffNoSimd EpEp;
typedef CalcForceEpSpQuadNoSimd EpSp;
typedef SearchNeighborEpEpNoSimd Nb;
#elif defined(REF_SIMD)
typedef CalcForceEpEpWithLinearCutoffSimd EpEp;
typedef CalcForceEpSpQuadSimd EpSp;
typedef SearchNeighborEpEpSimd Nb;
#else
#error "define REF_NOSIMD or REF_SIMD"
#endif

static void load_i(int ni, const double* xi, const double* rsi, EPISoft* epi) {
    for (int i = 0; i < ni; ++i) {
        epi[i].id = i;
        epi[i].pos = PS::F64vec(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]);
        epi[i].r_search = rsi[i];
        epi[i].rank_org = 0;
        epi[i].type = 1;
    }
}

extern "C" {

void ref_set_params(double eps, double r_out, double G) {
    EPISoft::eps = eps;
    EPISoft::r_out = r_out;
    ForceSoft::grav_const = G;
}

// EP-EP linear cutoff: acc, pot and n_ngb of ni i-particles against nj j-particles.
void ref_epep(int ni, const double* xi, const double* rsi, int nj, const double* xj, const double* mj,
              const double* rsj, double* acc, double* pot, long long* nnb) {
    EPISoft* epi = new EPISoft[ni > 0 ? ni : 1];
    EPJSoft* epj = new EPJSoft[nj > 0 ? nj : 1];
    ForceSoft* f = new ForceSoft[ni > 0 ? ni : 1];
    load_i(ni, xi, rsi, epi);
    for (int j = 0; j < nj; ++j) {
        epj[j].id = j;
        epj[j].mass = mj[j];
        epj[j].pos = PS::F64vec(xj[3 * j], xj[3 * j + 1], xj[3 * j + 2]);
        epj[j].r_search = rsj[j];
    }
    for (int i = 0; i < ni; ++i) f[i].clear();
    EpEp()(epi, ni, epj, nj, f);
    for (int i = 0; i < ni; ++i) {
        acc[3 * i] = f[i].acc.x;
        acc[3 * i + 1] = f[i].acc.y;
        acc[3 * i + 2] = f[i].acc.z;
        pot[i] = f[i].pot;
        nnb[i] = f[i].n_ngb;
    }
    delete[] epi;
    delete[] epj;
    delete[] f;
}

// EP-SP quadrupole; quad rows are (xx, yy, zz, xy, xz, yz).
void ref_epsp(int ni, const double* xi, int nj, const double* xj, const double* mj, const double* qj,
              double* acc, double* pot) {
    EPISoft* epi = new EPISoft[ni > 0 ? ni : 1];
    SPJSoft* spj = new SPJSoft[nj > 0 ? nj : 1];
    ForceSoft* f = new ForceSoft[ni > 0 ? ni : 1];
    double* zero = new double[ni > 0 ? ni : 1]();
    load_i(ni, xi, zero, epi);
    for (int j = 0; j < nj; ++j) {
        spj[j].mass = mj[j];
        spj[j].pos = PS::F64vec(xj[3 * j], xj[3 * j + 1], xj[3 * j + 2]);
        spj[j].quad.xx = qj[6 * j + 0];
        spj[j].quad.yy = qj[6 * j + 1];
        spj[j].quad.zz = qj[6 * j + 2];
        spj[j].quad.xy = qj[6 * j + 3];
        spj[j].quad.xz = qj[6 * j + 4];
        spj[j].quad.yz = qj[6 * j + 5];
    }
    for (int i = 0; i < ni; ++i) f[i].clear();
    EpSp()(epi, ni, spj, nj, f);
    for (int i = 0; i < ni; ++i) {
        acc[3 * i] = f[i].acc.x;
        acc[3 * i + 1] = f[i].acc.y;
        acc[3 * i + 2] = f[i].acc.z;
        pot[i] = f[i].pot;
    }
    delete[] epi;
    delete[] spj;
    delete[] f;
    delete[] zero;
}

// Neighbour search only.
void ref_nb(int ni, const double* xi, const double* rsi, int nj, const double* xj, const double* rsj,
            long long* nnb) {
    EPISoft* epi = new EPISoft[ni > 0 ? ni : 1];
    EPJSoft* epj = new EPJSoft[nj > 0 ? nj : 1];
    ForceSoft* f = new ForceSoft[ni > 0 ? ni : 1];
    load_i(ni, xi, rsi, epi);
    for (int j = 0; j < nj; ++j) {
        epj[j].id = j;
        epj[j].mass = 1.0;
        epj[j].pos = PS::F64vec(xj[3 * j], xj[3 * j + 1], xj[3 * j + 2]);
        epj[j].r_search = rsj[j];
    }
    for (int i = 0; i < ni; ++i) f[i].clear();
    Nb()(epi, ni, epj, nj, f);
    for (int i = 0; i < ni; ++i) nnb[i] = f[i].n_ngb;
    delete[] epi;
    delete[] epj;
    delete[] f;
}

#if defined(KDKDK_4TH) && defined(REF_NOSIMD)
// KDKDK_4TH gradient correction, EP-EP part (CalcCorrectEpEpWithLinearCutoffNoSimd,
// src/soft_force.hpp:89-122): acorr (no G) and the acc the functor writes
// (the i-particle's own acc), for ni i-particles against nj j-particles.
void ref_correct(int ni, const double* xi, const double* ai, int nj, const double* xj, const double* mj,
                 const double* aj, double* acorr, double* acc) {
    EPISoft* epi = new EPISoft[ni > 0 ? ni : 1];
    EPJSoft* epj = new EPJSoft[nj > 0 ? nj : 1];
    ForceSoft* f = new ForceSoft[ni > 0 ? ni : 1];
    for (int i = 0; i < ni; ++i) {
        epi[i].id = i;
        epi[i].pos = PS::F64vec(xi[3 * i], xi[3 * i + 1], xi[3 * i + 2]);
        epi[i].acc = PS::F64vec(ai[3 * i], ai[3 * i + 1], ai[3 * i + 2]);
        epi[i].r_search = 0.0;
        epi[i].rank_org = 0;
        epi[i].type = 1;
    }
    for (int j = 0; j < nj; ++j) {
        epj[j].id = j;
        epj[j].mass = mj[j];
        epj[j].pos = PS::F64vec(xj[3 * j], xj[3 * j + 1], xj[3 * j + 2]);
        epj[j].acc = PS::F64vec(aj[3 * j], aj[3 * j + 1], aj[3 * j + 2]);
        epj[j].r_search = 0.0;
    }
    for (int i = 0; i < ni; ++i) f[i].clear();
    CalcCorrectEpEpWithLinearCutoffNoSimd()(epi, ni, epj, nj, f);
    for (int i = 0; i < ni; ++i) {
        acorr[3 * i] = f[i].acorr.x;
        acorr[3 * i + 1] = f[i].acorr.y;
        acorr[3 * i + 2] = f[i].acorr.z;
        acc[3 * i] = f[i].acc.x;
        acc[3 * i + 1] = f[i].acc.y;
        acc[3 * i + 2] = f[i].acc.z;
    }
    delete[] epi;
    delete[] epj;
    delete[] f;
}
#endif

// Every walk of a multi-walk batch, OpenMP over walks with a dynamic schedule
// and buffers per thread, the way PeTar's tree walk calls its CPU functors
// (src/soft_force.hpp:365-373): the walk's EPJ and SPJ gathered from the
// shared arrays by its id lists (FDPS's interaction list), then EP-EP and
// EP-SP into one cleared Force per i.  For timing the reference CPU path over
// the same lists as the GPU kernels.
void ref_force_walks(int n_walk, const long long* epi_disp, const double* epi_pos, const double* epi_rs,
                     const long long* epj_disp, const int* id_epj, const long long* spj_disp, const int* id_spj,
                     const double* epj_pos, const double* epj_mass, const double* epj_rs, const double* spj_pos,
                     const double* spj_mass, const double* spj_quad, double* acc, double* pot, long long* nnb) {
#pragma omp parallel
    {
        std::vector<EPISoft> epi;
        std::vector<EPJSoft> epj;
        std::vector<SPJSoft> spj;
        std::vector<ForceSoft> f;
#pragma omp for schedule(dynamic, 1)
        for (int w = 0; w < n_walk; ++w) {
            const long long i0 = epi_disp[w], ni = epi_disp[w + 1] - i0;
            const long long e0 = epj_disp[w], ne = epj_disp[w + 1] - e0;
            const long long s0 = spj_disp[w], ns = spj_disp[w + 1] - s0;
            epi.resize(ni > 0 ? ni : 1);
            epj.resize(ne > 0 ? ne : 1);
            spj.resize(ns > 0 ? ns : 1);
            f.resize(ni > 0 ? ni : 1);
            load_i((int)ni, epi_pos + 3 * i0, epi_rs + i0, epi.data());
            for (long long j = 0; j < ne; ++j) {
                const int k = id_epj[e0 + j];
                epj[j].id = k;
                epj[j].mass = epj_mass[k];
                epj[j].pos = PS::F64vec(epj_pos[3 * k], epj_pos[3 * k + 1], epj_pos[3 * k + 2]);
                epj[j].r_search = epj_rs[k];
            }
            for (long long j = 0; j < ns; ++j) {
                const int k = id_spj[s0 + j];
                spj[j].mass = spj_mass[k];
                spj[j].pos = PS::F64vec(spj_pos[3 * k], spj_pos[3 * k + 1], spj_pos[3 * k + 2]);
                const double* q = spj_quad + 6 * k;
                spj[j].quad.xx = q[0];
                spj[j].quad.yy = q[1];
                spj[j].quad.zz = q[2];
                spj[j].quad.xy = q[3];
                spj[j].quad.xz = q[4];
                spj[j].quad.yz = q[5];
            }
            for (long long i = 0; i < ni; ++i) f[i].clear();
            if (ni > 0) {
                EpEp()(epi.data(), (int)ni, epj.data(), (int)ne, f.data());
                if (ns > 0) EpSp()(epi.data(), (int)ni, spj.data(), (int)ns, f.data());
            }
            for (long long i = 0; i < ni; ++i) {
                acc[3 * (i0 + i)] = f[i].acc.x;
                acc[3 * (i0 + i) + 1] = f[i].acc.y;
                acc[3 * (i0 + i) + 2] = f[i].acc.z;
                pot[i0 + i] = f[i].pot;
                nnb[i0 + i] = f[i].n_ngb;
            }
        }
    }
}

}  // extern "C"
