// mie.cu - Mie scattering amplitudes of a homogeneous sphere (host code).
//
// No reference counterpart: the reference's polarised E-field kernel is an
// empty stub (kernels.metal:1122-1187) and its host loads beam and phase
// tables from files that are not in the repository (MetalMC.m:286-312).  The
// amplitudes S1, S2 feed the E-field transport (efield.cu).
//
// The series is the classical Lorenz-Mie solution in the form of Bohren and
// Huffman, "Absorption and Scattering of Light by Small Particles" (1983),
// ch. 4 and appendix A, restated here from the mathematics:
//   * the logarithmic derivative D_n(mx) = psi_n'(mx)/psi_n(mx) by downward
//     recurrence D_{n-1} = n/(mx) - 1/(D_n + n/(mx)) from well above the
//     last term (it is unstable upward for absorbing spheres);
//   * the Riccati-Bessel functions psi_n(x) = x j_n(x) and chi_n(x) = -x y_n(x)
//     by upward recurrence f_n = (2n-1)/x f_{n-1} - f_{n-2}, xi = psi - i chi;
//   * a_n = ((D_n/m + n/x) psi_n - psi_{n-1}) / ((D_n/m + n/x) xi_n - xi_{n-1}),
//     b_n = ((m D_n + n/x) psi_n - psi_{n-1}) / ((m D_n + n/x) xi_n - xi_{n-1});
//   * angular functions pi_n, tau_n of mu = cos(theta) by their recurrences;
//   * S1 = sum (2n+1)/(n(n+1)) (a_n pi_n + b_n tau_n),
//     S2 = sum (2n+1)/(n(n+1)) (a_n tau_n + b_n pi_n);
//   * Q_sca = 2/x^2 sum (2n+1)(|a_n|^2 + |b_n|^2),
//     Q_ext = 2/x^2 sum (2n+1) Re(a_n + b_n),
//     g = 4/(x^2 Q_sca) sum [n(n+2)/(n+1) Re(a_n a*_{n+1} + b_n b*_{n+1})
//                             + (2n+1)/(n(n+1)) Re(a_n b*_n)].
// The series is summed to n_stop = x + 4 x^(1/3) + 2 terms (Wiscombe's
// criterion), in double precision.
#include <cmath>
#include <complex>
#include <vector>

#include "nmc_abi.h"

namespace {

using cd = std::complex<double>;

}  // namespace

extern "C" nmc_status nmc_mie(double x, double m_re, double m_im, int32_t n_angles, float* S, double* q_ext,
                              double* q_sca, double* g) {
  if (!(x > 0.0) || !std::isfinite(x) || x > 20000.0 || !(m_re > 0.0) || !std::isfinite(m_re) ||
      !(m_im >= 0.0) || !std::isfinite(m_im) || n_angles < 2 || n_angles > 1000000)
    return NMC_EINVAL;
  const cd m(m_re, m_im);
  const cd mx = m * x;
  const int nstop = (int)std::ceil(x + 4.0 * std::cbrt(x) + 2.0);
  const int nmx = (int)std::ceil(std::max((double)nstop, std::abs(mx))) + 16;
  std::vector<cd> D(nmx + 1);
  D[nmx] = cd(0.0, 0.0);
  for (int n = nmx; n >= 1; --n) {
    const cd r = (double)n / mx;
    D[n - 1] = r - 1.0 / (D[n] + r);
  }
  std::vector<cd> a(nstop + 2), b(nstop + 2);
  double psi_m1 = std::cos(x), psi_0 = std::sin(x);  // psi_{-1}, psi_0
  double chi_m1 = -std::sin(x), chi_0 = std::cos(x);
  cd xi_prev(psi_0, -chi_0);
  for (int n = 1; n <= nstop; ++n) {
    const double f = (2.0 * n - 1.0) / x;
    const double psi = f * psi_0 - psi_m1;
    const double chi = f * chi_0 - chi_m1;
    const cd xi(psi, -chi);
    const cd da = D[n] / m + (double)n / x;
    const cd db = m * D[n] + (double)n / x;
    a[n] = (da * psi - psi_0) / (da * xi - xi_prev);
    b[n] = (db * psi - psi_0) / (db * xi - xi_prev);
    psi_m1 = psi_0;
    psi_0 = psi;
    chi_m1 = chi_0;
    chi_0 = chi;
    xi_prev = xi;
  }
  a[nstop + 1] = b[nstop + 1] = cd(0.0, 0.0);
  double qs = 0.0, qe = 0.0, gs = 0.0;
  for (int n = 1; n <= nstop; ++n) {
    const double dn = n;
    qs += (2.0 * dn + 1.0) * (std::norm(a[n]) + std::norm(b[n]));
    qe += (2.0 * dn + 1.0) * (a[n].real() + b[n].real());
    gs += dn * (dn + 2.0) / (dn + 1.0) * (a[n] * std::conj(a[n + 1]) + b[n] * std::conj(b[n + 1])).real() +
          (2.0 * dn + 1.0) / (dn * (dn + 1.0)) * (a[n] * std::conj(b[n])).real();
  }
  const double x2 = x * x;
  if (q_sca) *q_sca = 2.0 / x2 * qs;
  if (q_ext) *q_ext = 2.0 / x2 * qe;
  if (g) *g = qs > 0.0 ? 2.0 * gs / qs : 0.0;  // (4/x^2) gs / Q_sca
  if (S) {
    const double pi_ = 3.14159265358979323846;
    for (int j = 0; j < n_angles; ++j) {
      const double mu = std::cos(pi_ * j / (n_angles - 1));
      double p_m1 = 0.0, p_0 = 1.0;  // pi_0, pi_1
      cd s1(0.0, 0.0), s2(0.0, 0.0);
      for (int n = 1; n <= nstop; ++n) {
        const double dn = n;
        const double p = p_0;  // pi_n
        const double t = dn * mu * p - (dn + 1.0) * p_m1;  // tau_n
        const double c = (2.0 * dn + 1.0) / (dn * (dn + 1.0));
        s1 += c * (a[n] * p + b[n] * t);
        s2 += c * (a[n] * t + b[n] * p);
        // pi_{n+1} = ((2n+1) mu pi_n - (n+1) pi_{n-1}) / n
        const double p_next = ((2.0 * dn + 1.0) * mu * p - (dn + 1.0) * p_m1) / dn;
        p_m1 = p;
        p_0 = p_next;
      }
      S[4 * j + 0] = (float)s1.real();
      S[4 * j + 1] = (float)s1.imag();
      S[4 * j + 2] = (float)s2.real();
      S[4 * j + 3] = (float)s2.imag();
    }
  }
  return NMC_OK;
}
