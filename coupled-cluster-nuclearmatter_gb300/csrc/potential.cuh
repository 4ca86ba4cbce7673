// Device potentials of the synthetic interactions (inline, shared by the kernels).
#pragma once

#include "common.cuh"
#include "devlayout.hpp"
#include "kernels.hpp"

namespace ccx {

namespace pot {
constexpr double kPi = 3.14159265358979;
constexpr double kHbarc = 197.326968;

__device__ inline double pauli_dot(int m1, int m2, int m3, int m4) {
  if (m1 == m3 && m2 == m4) return (double)(m1 * m2);
  if (m1 == m4 && m2 == m3 && m1 != m2) return 2.0;
  return 0.0;
}
__device__ inline double kd(int a, int b) { return a == b ? 1.0 : 0.0; }

// vmom_minnesota, chiral_module_andreas_with_delta.f90:8980-9111
__device__ inline double minnesota(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s) {
  if (O.nx[p] + O.nx[q] != O.nx[r] + O.nx[s] || O.ny[p] + O.ny[q] != O.ny[r] + O.ny[s] ||
      O.nz[p] + O.nz[q] != O.nz[r] + O.nz[s] || O.tz[p] + O.tz[q] != O.tz[r] + O.tz[s])
    return 0.0;
  const double q0 = 0.5 * (O.kx[p] - O.kx[q]) - 0.5 * (O.kx[r] - O.kx[s]);
  const double q1 = 0.5 * (O.ky[p] - O.ky[q]) - 0.5 * (O.ky[r] - O.ky[s]);
  const double q2v = 0.5 * (O.kz[p] - O.kz[q]) - 0.5 * (O.kz[r] - O.kz[s]);
  const double q2 = (q0 * q0 + q1 * q1) + q2v * q2v;
  double v0r, v0t, v0s, kr, kt, ks;
  if (P.f32_literals) {
    v0r = (double)200.0f; v0t = (double)178.0f; v0s = (double)91.85f;
    kr = (double)1.487f; kt = (double)0.639f; ks = (double)0.465f;
  } else {
    v0r = 200.0; v0t = 178.0; v0s = 91.85; kr = 1.487; kt = 0.639; ks = 0.465;
  }
  const double pi15 = kPi * sqrt(kPi);  // x^1.5 as x sqrt(x): no pow on the FP64 pipe
  double vr = v0r * pi15 * exp(-q2 / (4.0 * kr)) / (kr * sqrt(kr));
  double vt = -v0t * pi15 * exp(-q2 / (4.0 * kt)) / (kt * sqrt(kt));
  double vs = -v0s * pi15 * exp(-q2 / (4.0 * ks)) / (ks * sqrt(ks));
  const int m1 = O.sz[p], m2 = O.sz[q], m3 = O.sz[r], m4 = O.sz[s];
  const int t1 = O.tz[p], t2 = O.tz[q], t3 = O.tz[r], t4 = O.tz[s];
  const double dm = kd(m1, m3) * kd(m2, m4), dt = kd(t1, t3) * kd(t2, t4);
  const double tt = pauli_dot(t1, t2, t3, t4), ss = pauli_dot(m1, m2, m3, m4);
  vr = vr * (3.0 * dm * dt - tt * dm - ss * dt - tt * ss) / 8.0;
  vs = vs * (3.0 * dm * dt + tt * dm - 3.0 * ss * dt - tt * ss) / 16.0;
  vt = vt * (3.0 * dm * dt - 3.0 * tt * dm + ss * dt - tt * ss) / 16.0;
  return ((vs + vr) + vt) / O.volume;
}

constexpr double kLambda6 = 8.303765625e15;  // (450 MeV)^6 of the regulator exp(-(p/450)^6)

// nucleon mass of a pair's isospin projection (the relativity factor's mass)
__device__ inline double pair_mass(int t1, int t2) {
  const int tsum = (t1 + t2) / 2;
  return tsum < 0 ? 9.38272046000000046e+02 : (tsum == 0 ? 9.38918267117927371e+02 : 9.39565379000000007e+02);
}

__device__ inline cplx wsig(int ma, int mb, const double w[3]) {
  const int ia = ma > 0 ? 0 : 1, ib = mb > 0 ? 0 : 1;
  if (ia == 0 && ib == 0) return cplx(w[2], 0.0);
  if (ia == 1 && ib == 1) return cplx(-w[2], 0.0);
  if (ia == 0) return cplx(w[0], -w[1]);
  return cplx(w[0], w[1]);
}

// OPE + LO/NLO contacts in the operator form of chiral_pot (:5879-6301), regulated
// by freg (:3336-3351, n=3, Lambda=450 MeV), times hbarc^3/volume
__device__ inline cplx chiral_like(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s) {
  if (O.nx[p] + O.nx[q] != O.nx[r] + O.nx[s] || O.ny[p] + O.ny[q] != O.ny[r] + O.ny[s] ||
      O.nz[p] + O.nz[q] != O.nz[r] + O.nz[s] || O.tz[p] + O.tz[q] != O.tz[r] + O.tz[s])
    return cplx(0.0, 0.0);
  const double k1[3] = {O.kx[p] * kHbarc, O.ky[p] * kHbarc, O.kz[p] * kHbarc};
  const double k2[3] = {O.kx[q] * kHbarc, O.ky[q] * kHbarc, O.kz[q] * kHbarc};
  const double k3[3] = {O.kx[r] * kHbarc, O.ky[r] * kHbarc, O.kz[r] * kHbarc};
  const double k4[3] = {O.kx[s] * kHbarc, O.ky[s] * kHbarc, O.kz[s] * kHbarc};
  double pr[3], pp[3], km[3], qt[3], qxk[3];
  for (int d = 0; d < 3; ++d) {
    pr[d] = 0.5 * (k1[d] - k2[d]);
    pp[d] = 0.5 * (k3[d] - k4[d]);
    km[d] = 0.5 * (pr[d] + pp[d]);
    qt[d] = pr[d] - pp[d];
  }
  const double p2 = (pr[0] * pr[0] + pr[1] * pr[1]) + pr[2] * pr[2];
  const double pp2 = (pp[0] * pp[0] + pp[1] * pp[1]) + pp[2] * pp[2];
  const double km2 = (km[0] * km[0] + km[1] * km[1]) + km[2] * km[2];
  const double q2 = (qt[0] * qt[0] + qt[1] * qt[1]) + qt[2] * qt[2];
  qxk[0] = qt[1] * km[2] - qt[2] * km[1];
  qxk[1] = qt[2] * km[0] - qt[0] * km[2];
  qxk[2] = qt[0] * km[1] - qt[1] * km[0];
  const int m1 = O.sz[p], m2 = O.sz[q], m3 = O.sz[r], m4 = O.sz[s];
  const int t1 = O.tz[p], t2 = O.tz[q], t3 = O.tz[r], t4 = O.tz[s];
  const int tsum = (t1 + t2) / 2;
  const double mn = tsum < 0 ? 9.38272046000000046e+02 : (tsum == 0 ? 9.38918267117927371e+02 : 9.39565379000000007e+02);
  const double rel = mn / sqrt(sqrt((mn * mn + p2) * (mn * mn + pp2)));
  const double dm = kd(m1, m3) * kd(m2, m4), dt = kd(t1, t3) * kd(t2, t4);
  const double tt = pauli_dot(t1, t2, t3, t4), ss = pauli_dot(m1, m2, m3, m4);
  const cplx sq = wsig(m1, m3, qt) * wsig(m2, m4, qt);
  const cplx sk = wsig(m1, m3, km) * wsig(m2, m4, km);
  const cplx mi(0.0, -0.5);
  const cplx sl = mi * wsig(m1, m3, qxk) * kd(m2, m4) + mi * wsig(m2, m4, qxk) * kd(m1, m3);
  const double c2 = (1.27 * 1.27) / (4.0 * 92.4 * 92.4);
  const double ope = -1.0 * c2 / (q2 + 138.0 * 138.0);
  const cplx vlo = (ope * tt) * sq;
  const double *c = P.lec;
  const cplx cont_lo = cplx(c[0] * dm * dt + c[1] * ss * dt, 0.0);
  const cplx cont_nlo = cplx(c[2] * q2 * dm * dt + c[3] * km2 * dm * dt + c[4] * q2 * ss * dt + c[5] * km2 * ss * dt, 0.0) +
                        (c[6] * dt) * sl + (c[7] * dt) * sq + (c[8] * dt) * sk;
  const double l2n = kLambda6;
  const double freg = exp(-((p2 * p2) * p2 / l2n + (pp2 * pp2) * pp2 / l2n));
  const cplx vdir = ((vlo + cont_lo) + cont_nlo) * (rel * freg);
  return (kHbarc * kHbarc * kHbarc) * vdir * (1.0 / O.volume);
}

// The chiral-like element factorised as m F(pq) F(rs) core(p, q, r, s): the relativity
// factor m / ((m^2 + p^2)(m^2 + p'^2))^(1/4) and the regulator exp(-(p^6 + p'^6)/L^6)
// depend on the relative momentum of one pair each, and both are unchanged when r and s
// swap, so an antisymmetrised element is m F(pq) F(rs) (core(pqrs) - core(pqsr)).
// F(pq) is evaluated once per pair; the core per element holds no transcendental.
__device__ inline double chiral_pair_factor(const DevOrbits &O, int p, int q) {
  const double x = 0.5 * (O.kx[p] * kHbarc - O.kx[q] * kHbarc), y = 0.5 * (O.ky[p] * kHbarc - O.ky[q] * kHbarc);
  const double z = 0.5 * (O.kz[p] * kHbarc - O.kz[q] * kHbarc);
  const double p2 = (x * x + y * y) + z * z;
  const double mn = pair_mass(O.tz[p], O.tz[q]);
  return exp(-(p2 * p2) * p2 / kLambda6) / sqrt(sqrt(mn * mn + p2));
}
__device__ inline cplx chiral_core(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s) {
  if (O.nx[p] + O.nx[q] != O.nx[r] + O.nx[s] || O.ny[p] + O.ny[q] != O.ny[r] + O.ny[s] ||
      O.nz[p] + O.nz[q] != O.nz[r] + O.nz[s] || O.tz[p] + O.tz[q] != O.tz[r] + O.tz[s])
    return cplx(0.0, 0.0);
  double pr[3], pp[3], km[3], qt[3], qxk[3];
  const double k1[3] = {O.kx[p], O.ky[p], O.kz[p]}, k2[3] = {O.kx[q], O.ky[q], O.kz[q]};
  const double k3[3] = {O.kx[r], O.ky[r], O.kz[r]}, k4[3] = {O.kx[s], O.ky[s], O.kz[s]};
  for (int d = 0; d < 3; ++d) {
    pr[d] = 0.5 * (k1[d] * kHbarc - k2[d] * kHbarc);
    pp[d] = 0.5 * (k3[d] * kHbarc - k4[d] * kHbarc);
    km[d] = 0.5 * (pr[d] + pp[d]);
    qt[d] = pr[d] - pp[d];
  }
  const double km2 = (km[0] * km[0] + km[1] * km[1]) + km[2] * km[2];
  const double q2 = (qt[0] * qt[0] + qt[1] * qt[1]) + qt[2] * qt[2];
  qxk[0] = qt[1] * km[2] - qt[2] * km[1];
  qxk[1] = qt[2] * km[0] - qt[0] * km[2];
  qxk[2] = qt[0] * km[1] - qt[1] * km[0];
  const int m1 = O.sz[p], m2 = O.sz[q], m3 = O.sz[r], m4 = O.sz[s];
  const int t1 = O.tz[p], t2 = O.tz[q], t3 = O.tz[r], t4 = O.tz[s];
  const double dm = kd(m1, m3) * kd(m2, m4), dt = kd(t1, t3) * kd(t2, t4);
  const double tt = pauli_dot(t1, t2, t3, t4), ss = pauli_dot(m1, m2, m3, m4);
  const cplx sq = wsig(m1, m3, qt) * wsig(m2, m4, qt);
  const cplx sk = wsig(m1, m3, km) * wsig(m2, m4, km);
  const cplx mi(0.0, -0.5);
  const cplx sl = mi * wsig(m1, m3, qxk) * kd(m2, m4) + mi * wsig(m2, m4, qxk) * kd(m1, m3);
  const double c2 = (1.27 * 1.27) / (4.0 * 92.4 * 92.4);
  const double ope = -1.0 * c2 / (q2 + 138.0 * 138.0);
  const cplx vlo = (ope * tt) * sq;
  const double *c = P.lec;
  const cplx cont_lo = cplx(c[0] * dm * dt + c[1] * ss * dt, 0.0);
  const cplx cont_nlo = cplx(c[2] * q2 * dm * dt + c[3] * km2 * dm * dt + c[4] * q2 * ss * dt + c[5] * km2 * ss * dt, 0.0) +
                        (c[6] * dt) * sl + (c[7] * dt) * sq + (c[8] * dt) * sk;
  return (kHbarc * kHbarc * kHbarc) * ((vlo + cont_lo) + cont_nlo) * (1.0 / O.volume);
}
// antisymmetrised chiral-like element from the pair factors fpq = F(pq), frs = F(rs)
__device__ inline cplx chiral_anti_factored(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s,
                                            double fpq, double frs) {
  const double w = pair_mass(O.tz[p], O.tz[q]) * fpq * frs;
  return (chiral_core(O, P, p, q, r, s) - chiral_core(O, P, p, q, s, r)) * w;
}

template <typename S> __device__ S vbare(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s);
template <> __device__ inline double vbare<double>(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s) {
  return minnesota(O, P, p, q, r, s);
}
template <> __device__ inline cplx vbare<cplx>(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s) {
  if (P.kind == 1) return chiral_like(O, P, p, q, r, s);
  return cplx(minnesota(O, P, p, q, r, s), 0.0);
}
template <typename S> __device__ inline S vanti(const DevOrbits &O, const DevPotential &P, int p, int q, int r, int s) {
  return vbare<S>(O, P, p, q, r, s) - vbare<S>(O, P, p, q, s, r);
}
}  // namespace pot

}  // namespace ccx
