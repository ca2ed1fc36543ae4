/* FP64 CPU oracle for the long-range soft-force path.
 *
 * TEST INFRASTRUCTURE ONLY: tests, the smoke check and the CPU-baseline leg of
 * the benchmark use this to check and time the GPU kernels.  Nothing in the
 * product links or calls it.
 *
 * It restates, per interaction list, the reference's FP64 functors:
 *   EP-EP linear cutoff + neighbour count: src/soft_force.hpp:38-87
 *     (CalcForceEpEpWithLinearCutoffNoSimd)
 *   EP-SP quadrupole:                      src/soft_force.hpp:160-200
 *     (CalcForceEpSpQuadNoSimd)
 * with the neighbour test of the GPU functor it replaces,
 * src/force_gpu_cuda.cu:62-64: r2 + eps2 < max(rs_i, rs_j)^2 (self included,
 * no mass or type filtering).  nnb_with_eps = 0 selects the NoSimd form
 * r2 < max(rs_i, rs_j)^2 instead; the two agree when eps = 0.
 *
 * Every expression keeps the reference's evaluation order and is compiled
 * with -ffp-contract=off so results do not depend on the host's FMA support.
 * Parity is pinned against the reference's own functors, compiled from the
 * reference sources by oracle/ref/build_ref.sh, through the golden fixtures in
 * tests/golden/.
 */
#include <math.h>
#include <stdint.h>

static inline double dmax(double a, double b) { return a > b ? a : b; }

/* One walk's EP-EP sum for i-particle (xi, rsi) over its EPJ list.
 * Follows src/soft_force.hpp:53-71. */
static void epep_one(const double xi[3], double rsi, const double *epj_pos, const double *epj_mass,
                     const double *epj_rs, const int32_t *ids, int64_t nj, double eps2, double r_out2,
                     int nnb_with_eps, double ai[3], double *poti, int64_t *nnb) {
    double ax = 0.0, ay = 0.0, az = 0.0, p = 0.0;
    int64_t n = 0;
    for (int64_t k = 0; k < nj; ++k) {
        const int64_t j = ids[k];
        const double rx = xi[0] - epj_pos[3 * j + 0];
        const double ry = xi[1] - epj_pos[3 * j + 1];
        const double rz = xi[2] - epj_pos[3 * j + 2];
        const double r2 = rx * rx + ry * ry + rz * rz;
        const double r2_eps = r2 + eps2;
        const double r_search = dmax(rsi, epj_rs[j]);
        const double r2_test = nnb_with_eps ? r2_eps : r2;
        if (r2_test < r_search * r_search) n++;
        const double r2_tmp = (r2_eps > r_out2) ? r2_eps : r_out2;
        const double r_inv = 1.0 / sqrt(r2_tmp);
        const double m_r = epj_mass[j] * r_inv;
        const double m_r3 = m_r * r_inv * r_inv;
        ax -= m_r3 * rx;
        ay -= m_r3 * ry;
        az -= m_r3 * rz;
        p -= m_r;
    }
    ai[0] = ax;
    ai[1] = ay;
    ai[2] = az;
    *poti = p;
    *nnb = n;
}

/* One walk's EP-SP quadrupole sum.  Follows src/soft_force.hpp:174-195;
 * quad is (xx, yy, zz, xy, xz, yz), the raw second moment about the centre of
 * mass. */
static void epsp_one(const double xi[3], const double *spj_pos, const double *spj_mass,
                     const double *spj_quad, const int32_t *ids, int64_t nj, double eps2, double ai[3],
                     double *poti) {
    double ax = 0.0, ay = 0.0, az = 0.0, p = 0.0;
    for (int64_t k = 0; k < nj; ++k) {
        const int64_t j = ids[k];
        const double mj = spj_mass[j];
        const double rx = xi[0] - spj_pos[3 * j + 0];
        const double ry = xi[1] - spj_pos[3 * j + 1];
        const double rz = xi[2] - spj_pos[3 * j + 2];
        const double r2 = rx * rx + ry * ry + rz * rz + eps2;
        const double *q = spj_quad + 6 * j;
        const double qxx = q[0], qyy = q[1], qzz = q[2], qxy = q[3], qxz = q[4], qyz = q[5];
        const double tr = qxx + qyy + qzz;
        const double qrx = qxx * rx + qxy * ry + qxz * rz;
        const double qry = qyy * ry + qyz * rz + qxy * rx;
        const double qrz = qzz * rz + qxz * rx + qyz * ry;
        const double qrr = qrx * rx + qry * ry + qrz * rz;
        const double r_inv = 1.0f / sqrt(r2);
        const double r2_inv = r_inv * r_inv;
        const double r3_inv = r2_inv * r_inv;
        const double r5_inv = r2_inv * r3_inv * 1.5;
        const double qrr_r5 = r5_inv * qrr;
        const double qrr_r7 = r2_inv * qrr_r5;
        const double A = mj * r3_inv - tr * r5_inv + 5 * qrr_r7;
        const double B = -2.0 * r5_inv;
        ax -= A * rx + B * qrx;
        ay -= A * ry + B * qry;
        az -= A * rz + B * qrz;
        p -= mj * r_inv - 0.5 * tr * r3_inv + qrr_r5;
    }
    ai[0] = ax;
    ai[1] = ay;
    ai[2] = az;
    *poti = p;
}

/* Full multi-walk evaluation.  Outputs are per EPI row (walk order):
 *   acc[3*i], pot[i]       : G*ai_ep + G*ai_sp, as the two functors accumulate
 *                            into one ForceSoft (src/soft_force.hpp:73,77,196-197)
 *   nnb[i]                 : neighbour count
 *   acc_ep/pot_ep/acc_sp/pot_sp (each may be NULL): the separate G-scaled parts.
 * walk_rcut2 (may be NULL) overrides r_out^2 per walk for independent clusters. */
void oracle_force(int64_t n_walk, const int64_t *epi_disp, const double *epi_pos, const double *epi_rs,
                  const double *epj_pos, const double *epj_mass, const double *epj_rs,
                  const double *spj_pos, const double *spj_mass, const double *spj_quad,
                  const int64_t *epj_disp, const int32_t *id_epj, const int64_t *spj_disp,
                  const int32_t *id_spj, double eps2, double rcut2, double G, const double *walk_rcut2,
                  int nnb_with_eps, double *acc, double *pot, int64_t *nnb, double *acc_ep,
                  double *pot_ep, double *acc_sp, double *pot_sp) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t w = 0; w < n_walk; ++w) {
        const double r_out2 = walk_rcut2 ? walk_rcut2[w] : rcut2;
        for (int64_t i = epi_disp[w]; i < epi_disp[w + 1]; ++i) {
            const double *xi = epi_pos + 3 * i;
            double ae[3], pe, as[3], ps;
            int64_t n;
            epep_one(xi, epi_rs[i], epj_pos, epj_mass, epj_rs, id_epj + epj_disp[w],
                     epj_disp[w + 1] - epj_disp[w], eps2, r_out2, nnb_with_eps, ae, &pe, &n);
            epsp_one(xi, spj_pos, spj_mass, spj_quad, id_spj + spj_disp[w], spj_disp[w + 1] - spj_disp[w],
                     eps2, as, &ps);
            double f[3], p;
            for (int d = 0; d < 3; ++d) f[d] = 0.0 + G * ae[d];
            p = 0.0 + G * pe;
            for (int d = 0; d < 3; ++d) f[d] += G * as[d];
            p += G * ps;
            for (int d = 0; d < 3; ++d) acc[3 * i + d] = f[d];
            pot[i] = p;
            nnb[i] = n;
            if (acc_ep) for (int d = 0; d < 3; ++d) acc_ep[3 * i + d] = G * ae[d];
            if (pot_ep) pot_ep[i] = G * pe;
            if (acc_sp) for (int d = 0; d < 3; ++d) acc_sp[3 * i + d] = G * as[d];
            if (pot_sp) pot_sp[i] = G * ps;
        }
    }
}

/* Global neighbour count over all particles (no tree): for each i, the number
 * of j with |xi-xj|^2 + eps2 < max(rs_i, rs_j)^2, self included. */
void oracle_nnb_global(int64_t n, const double *pos, const double *rs, double eps2, int64_t *nnb) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        for (int64_t j = 0; j < n; ++j) {
            const double rx = pos[3 * i + 0] - pos[3 * j + 0];
            const double ry = pos[3 * i + 1] - pos[3 * j + 1];
            const double rz = pos[3 * i + 2] - pos[3 * j + 2];
            const double r2 = rx * rx + ry * ry + rz * rz + eps2;
            const double r_search = dmax(rs[i], rs[j]);
            if (r2 < r_search * r_search) c++;
        }
        nnb[i] = c;
    }
}

/* Direct N^2 FP64 sum of unsoftened gravity with the same linear cutoff, for
 * the truth side of force-error statistics (no tree, no multipoles). */
void oracle_direct(int64_t n_target, const int64_t *target, int64_t n, const double *pos,
                   const double *mass, double eps2, double rcut2, double G, double *acc, double *pot) {
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t t = 0; t < n_target; ++t) {
        const int64_t i = target[t];
        double ax = 0, ay = 0, az = 0, p = 0;
        for (int64_t j = 0; j < n; ++j) {
            const double rx = pos[3 * i + 0] - pos[3 * j + 0];
            const double ry = pos[3 * i + 1] - pos[3 * j + 1];
            const double rz = pos[3 * i + 2] - pos[3 * j + 2];
            const double r2 = rx * rx + ry * ry + rz * rz + eps2;
            const double r2c = r2 > rcut2 ? r2 : rcut2;
            const double ri = 1.0 / sqrt(r2c);
            const double mr = mass[j] * ri;
            const double mr3 = mr * ri * ri;
            ax -= mr3 * rx;
            ay -= mr3 * ry;
            az -= mr3 * rz;
            p -= mr;
        }
        acc[3 * t + 0] = G * ax;
        acc[3 * t + 1] = G * ay;
        acc[3 * t + 2] = G * az;
        pot[t] = G * p;
    }
}

/* ---- Changeover functions (src/changeover.hpp, default build: the
 * potential-based W of the #else branch, INTEGRATED_CUTOFF_FUNCTION unset) ---- */
typedef struct {
    double r_in, r_out, norm, coff, pot_off;
} co_t;

/* ChangeOver::setR(r_in, r_out), src/changeover.hpp:64-75. */
static co_t co_make(double r_in, double r_out) {
    co_t c;
    c.r_in = r_in;
    c.r_out = r_out;
    c.norm = 1.0 / (r_out - r_in);
    c.coff = (r_out - r_in) / (r_out + r_in);
    c.pot_off = (1.0 + c.coff) / r_out;
    return c;
}

/* calcPotW, src/changeover.hpp:294-309. */
static double co_potw(const co_t *c, double dr) {
    const double x = (dr - c->r_in) * c->norm;
    double k = 1.0;
    if (x >= 1.0) {
        k = c->pot_off * dr;
    } else if (x > 0.0) {
        const double x2 = x * x;
        const double x3 = x2 * x;
        const double x5 = x2 * x3;
        k -= c->coff * x5 * (5.0 * x3 - 20.0 * x2 + 28.0 * x - 14.0);
    }
    return k;
}

/* calcAcc0W, src/changeover.hpp:318-334. */
static double co_acc0w(const co_t *c, double dr) {
    double x = (dr - c->r_in) * c->norm;
    x = (x < 1.0) ? x : 1.0;
    x = (x > 0.0) ? x : 0.0;
    const double x_1 = x - 1;
    const double x_2 = x_1 * x_1;
    const double x_4 = x_2 * x_2;
    const double x2 = x * x;
    const double x3 = x2 * x;
    const double x4 = x2 * x2;
    return x_4 * (1.0 + 4.0 * x + 10.0 * x2 + 20.0 * x3 + 35.0 * c->coff * x4);
}

/* calcAcc0WTwo / calcPotWTwo pick the changeover with the larger r_out, the
 * second one on a tie (src/changeover.hpp:364-375). */
static const co_t *co_pick(const co_t *a, const co_t *b) { return a->r_out > b->r_out ? a : b; }

void oracle_co_w(int64_t n, const double *r_in, const double *r_out, const double *dr, double *acc0w,
                 double *potw) {
    for (int64_t i = 0; i < n; ++i) {
        const co_t c = co_make(r_in[i], r_out[i]);
        acc0w[i] = co_acc0w(&c, dr[i]);
        potw[i] = co_potw(&c, dr[i]);
    }
}

void oracle_co_w_two(int64_t n, const double *r_in1, const double *r_out1, const double *r_in2,
                     const double *r_out2, const double *dr, double *acc0w, double *potw) {
    for (int64_t i = 0; i < n; ++i) {
        const co_t a = co_make(r_in1[i], r_out1[i]);
        const co_t b = co_make(r_in2[i], r_out2[i]);
        const co_t *c = co_pick(&a, &b);
        acc0w[i] = co_acc0w(c, dr[i]);
        potw[i] = co_potw(c, dr[i]);
    }
}

/* Soft force of each EPI with the changeover correction of its tree
 * neighbours applied, as PeTar composes it for one force evaluation:
 *   1. the linear-cutoff EP-EP and EP-SP sums (oracle_force); FPSoft copies
 *      ForceSoft.pot into pot_tot and pot_soft (src/soft_ptcl.hpp:84-95);
 *   2. the self-potential G m / r_out for particles with a self term
 *      (src/hard.hpp:1663-1674; self_mass is that mass, 0 for none);
 *   3. for every other EPJ of the walk's list within the neighbour radius
 *      (the count's test: |dx|^2 + eps2 < max(rs_i, rs_j)^2, which is the tree
 *      search's for eps = 0), calcAccPotShortWithLinearCutoff for EPJSoft,
 *      FP64 branch (src/hard.hpp:1404-1480): the cutoff term is replaced by
 *      the changeover force k = 1 - W_acc(r) of the pair's larger r_out, and
 *      the potentials follow the artificial-particle status of j (single:
 *      status == 0 and mass_backup == 0; member: status < 0, potential from
 *      mass_backup; otherwise the pair's potential is removed).
 * r_out of the correction is the walk's cutoff radius (EPISoft::r_out). */
void oracle_force_changeover(int64_t n_walk, const int64_t *epi_disp, const double *epi_pos,
                             const double *epi_rs, const double *epj_pos, const double *epj_mass,
                             const double *epj_rs, const double *spj_pos, const double *spj_mass,
                             const double *spj_quad, const int64_t *epj_disp, const int32_t *id_epj,
                             const int64_t *spj_disp, const int32_t *id_spj, double eps2, double rcut2, double G,
                             const double *walk_rcut2, const int64_t *epi_id, const double *epi_rin,
                             const double *epi_rout, const double *epi_mself, const int64_t *epj_id,
                             const double *epj_rin, const double *epj_rout, const double *epj_mbk,
                             const double *epj_status, double *acc, double *pot_tot, double *pot_soft,
                             int64_t *nnb) {
    oracle_force(n_walk, epi_disp, epi_pos, epi_rs, epj_pos, epj_mass, epj_rs, spj_pos, spj_mass, spj_quad,
                 epj_disp, id_epj, spj_disp, id_spj, eps2, rcut2, G, walk_rcut2, 1, acc, pot_tot, nnb, 0, 0, 0, 0);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t w = 0; w < n_walk; ++w) {
        const double r_out2 = walk_rcut2 ? walk_rcut2[w] : rcut2;
        const double r_out = sqrt(r_out2);
        for (int64_t i = epi_disp[w]; i < epi_disp[w + 1]; ++i) {
            const double *xi = epi_pos + 3 * i;
            const co_t ci = co_make(epi_rin[i], epi_rout[i]);
            double ax = acc[3 * i + 0], ay = acc[3 * i + 1], az = acc[3 * i + 2];
            double pt = pot_tot[i], ps = pot_tot[i];
            if (epi_mself[i] != 0.0) {
                const double pot_cor = G * epi_mself[i] / r_out;
                pt += pot_cor;
                ps += pot_cor;
            }
            for (int64_t k = epj_disp[w]; k < epj_disp[w + 1]; ++k) {
                const int64_t j = id_epj[k];
                if (epj_id[j] == epi_id[i]) continue;
                const double rx = xi[0] - epj_pos[3 * j + 0];
                const double ry = xi[1] - epj_pos[3 * j + 1];
                const double rz = xi[2] - epj_pos[3 * j + 2];
                const double dr2 = rx * rx + ry * ry + rz * rz;
                const double dr2_eps = dr2 + eps2;
                const double r_search = dmax(epi_rs[i], epj_rs[j]);
                if (!(dr2_eps < r_search * r_search)) continue;
                const double drinv = 1.0 / sqrt(dr2_eps);
                double gmor = G * epj_mass[j] * drinv;
                const double drinv2 = drinv * drinv;
                const double gmor3 = gmor * drinv2;
                const double dr_eps = drinv * dr2_eps;
                const co_t cj = co_make(epj_rin[j], epj_rout[j]);
                const co_t *c = co_pick(&ci, &cj);
                const double kacc = 1.0 - co_acc0w(c, dr_eps);
                const double dr2_max = (dr2_eps > r_out2) ? dr2_eps : r_out2;
                const double drinv_max = 1.0 / sqrt(dr2_max);
                const double gmor_max = G * epj_mass[j] * drinv_max;
                const double drinv2_max = drinv_max * drinv_max;
                const double gmor3_max = gmor_max * drinv2_max;
                const double s = gmor3 * kacc - gmor3_max;
                ax -= s * rx;
                ay -= s * ry;
                az -= s * rz;
                const double kpot = 1.0 - co_potw(c, dr_eps);
                const double status = epj_status[j], mbk = epj_mbk[j];
                if (status == 0.0 && mbk == 0.0) {
                    ps -= gmor * kpot - gmor_max;
                    pt -= (gmor - gmor_max);
                } else if (status < 0.0) {
                    gmor = G * mbk * drinv;
                    ps -= gmor * kpot - gmor_max;
                    pt -= (gmor - gmor_max);
                } else {
                    ps += gmor_max;
                    pt += gmor_max;
                }
            }
            acc[3 * i + 0] = ax;
            acc[3 * i + 1] = ay;
            acc[3 * i + 2] = az;
            pot_tot[i] = pt;
            pot_soft[i] = ps;
        }
    }
}

/* KDKDK_4TH gradient-correction pass (src/petar.hpp:1123-1140): per walk,
 * CalcCorrectEpEpWithLinearCutoffNoSimd (src/soft_force.hpp:89-122) over the
 * EPJ list, then the quadrupole EP-SP force functor (src/soft_force.hpp:
 * 160-200), accumulated into one cleared ForceSoft as FDPS does:
 *   acorr = 2 sum_j -m_j/r^3 (da - 3 (dr.da)/r^2 dr)   (no G; r = max(r, r_out))
 *   acc   = acc_i + G acc_sp,   pot = G pot_sp. */
void oracle_gradient(int64_t n_walk, const int64_t *epi_disp, const double *epi_pos, const double *epi_acc,
                     const double *epj_pos, const double *epj_mass, const double *epj_acc,
                     const double *spj_pos, const double *spj_mass, const double *spj_quad,
                     const int64_t *epj_disp, const int32_t *id_epj, const int64_t *spj_disp,
                     const int32_t *id_spj, double eps2, double rcut2, double G, const double *walk_rcut2,
                     double *acorr, double *acc, double *pot) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t w = 0; w < n_walk; ++w) {
        const double r_out2 = walk_rcut2 ? walk_rcut2[w] : rcut2;
        for (int64_t i = epi_disp[w]; i < epi_disp[w + 1]; ++i) {
            const double *xi = epi_pos + 3 * i;
            const double *ai = epi_acc + 3 * i;
            double cx = 0.0, cy = 0.0, cz = 0.0;
            for (int64_t k = epj_disp[w]; k < epj_disp[w + 1]; ++k) {
                const int64_t j = id_epj[k];
                const double drx = xi[0] - epj_pos[3 * j + 0];
                const double dry = xi[1] - epj_pos[3 * j + 1];
                const double drz = xi[2] - epj_pos[3 * j + 2];
                const double dax = ai[0] - epj_acc[3 * j + 0];
                const double day = ai[1] - epj_acc[3 * j + 1];
                const double daz = ai[2] - epj_acc[3 * j + 2];
                const double r2 = drx * drx + dry * dry + drz * drz + eps2;
                const double drda = drx * dax + dry * day + drz * daz;
                const double r2_tmp = (r2 > r_out2) ? r2 : r_out2;
                const double r_inv = 1.0 / sqrt(r2_tmp);
                const double r2_inv = r_inv * r_inv;
                const double m_r = epj_mass[j] * r_inv;
                const double m_r3 = m_r * r2_inv;
                const double alpha = 3.0 * drda * r2_inv;
                cx -= m_r3 * (dax - alpha * drx);
                cy -= m_r3 * (day - alpha * dry);
                cz -= m_r3 * (daz - alpha * drz);
            }
            acorr[3 * i + 0] = 0.0 + 2.0 * cx;
            acorr[3 * i + 1] = 0.0 + 2.0 * cy;
            acorr[3 * i + 2] = 0.0 + 2.0 * cz;
            double as[3], ps;
            epsp_one(xi, spj_pos, spj_mass, spj_quad, id_spj + spj_disp[w], spj_disp[w + 1] - spj_disp[w], eps2,
                     as, &ps);
            for (int d = 0; d < 3; ++d) acc[3 * i + d] = ai[d] + G * as[d];
            pot[i] = 0.0 + G * ps;
        }
    }
}
