// Exposes the reference's changeover functions (src/changeover.hpp) through a
// C interface, compiled from the reference source by oracle/ref/build_ref.sh.
// The default build of PeTar leaves INTEGRATED_CUTOFF_FUNCTION undefined
// (Makefile.in), so the potential-based W functions are the ones compiled.
#include "changeover.hpp"

extern "C" {

// W_acc and W_pot of one changeover (r_in, r_out) at separation dr
// (ChangeOver::setR(r_in, r_out), calcAcc0W, calcPotW).
void ref_co_w(int n, const double* r_in, const double* r_out, const double* dr, double* acc0w, double* potw) {
    for (int i = 0; i < n; ++i) {
        ChangeOver co;
        co.setR(r_in[i], r_out[i]);
        acc0w[i] = co.calcAcc0W(dr[i]);
        potw[i] = co.calcPotW(dr[i]);
    }
}

// The pair forms: the changeover with the larger r_out (calcAcc0WTwo, calcPotWTwo).
void ref_co_w_two(int n, const double* r_in1, const double* r_out1, const double* r_in2, const double* r_out2,
                  const double* dr, double* acc0w, double* potw) {
    for (int i = 0; i < n; ++i) {
        ChangeOver a, b;
        a.setR(r_in1[i], r_out1[i]);
        b.setR(r_in2[i], r_out2[i]);
        acc0w[i] = ChangeOver::calcAcc0WTwo(a, b, dr[i]);
        potw[i] = ChangeOver::calcPotWTwo(a, b, dr[i]);
    }
}

// Mass-scaled radii (setR(m_fac, r_in, r_out)): r * max(m_fac^(1/3), 1).
void ref_co_setr_mfac(int n, const double* m_fac, const double* r_in, const double* r_out, double* r_in_o,
                      double* r_out_o) {
    for (int i = 0; i < n; ++i) {
        ChangeOver co;
        co.setR(m_fac[i], r_in[i], r_out[i]);
        r_in_o[i] = co.getRin();
        r_out_o[i] = co.getRout();
    }
}

}  // extern "C"
