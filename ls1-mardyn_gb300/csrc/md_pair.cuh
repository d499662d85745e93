// md_pair.cuh -- site-site interaction bodies, templated on the arithmetic
// type (double for the FP64 kernel, float for the mixed kernel).
//
// Physics of VectorizedCellProcessor::_loopBodyLJ/Charge/ChargeDipole/Dipole/
// ChargeQuadrupole/DipoleQuadrupole/Quadrupole
// (src/particleContainer/adapter/VectorizedCellProcessor.cpp:171-792), seen
// from one side: every function returns the force f on site "a" (the site of
// the thread's own molecule), the torque T on a's orientation, the virial
// contribution m_d o f (m_d = molecule-centre distance) and the pair energy
// u (counted by the caller on one side of the pair only).
#pragma once
#include "md_device.cuh"

namespace md {

// FP32: the hardware approximations (about 1 ulp), which the FP32 pair
// arithmetic tolerates; FP64: IEEE division and square root.
__device__ __forceinline__ float rcp_approx_f(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float sqrt_approx_f(float x) {
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
template <typename Real> __device__ __forceinline__ Real rcp_(Real x);
template <> __device__ __forceinline__ float rcp_<float>(float x) { return rcp_approx_f(x); }
template <> __device__ __forceinline__ double rcp_<double>(double x) { return 1.0 / x; }
template <typename Real> __device__ __forceinline__ Real sqrt_(Real x);
template <> __device__ __forceinline__ float sqrt_<float>(float x) { return sqrt_approx_f(x); }
template <> __device__ __forceinline__ double sqrt_<double>(double x) { return sqrt(x); }

template <typename Real>
__device__ __forceinline__ Real dot3(const Real* a, const Real* b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }

// LJ-12-6 (VCP.cpp:171-224): d = site distance, md = centre distance.
// u = eps24 (lj12 - lj6) + shift6 (the reference sums u and divides by 6).
template <typename Real>
__device__ __forceinline__ void lj_pair(const Real* d, const Real* md, Real r2, Real eps24, Real sig2, Real shift6,
                                        Real* f, Real* V, Real& u) {
    Real r2inv = rcp_<Real>(r2);
    Real lj2 = sig2 * r2inv;
    Real lj6 = lj2 * lj2 * lj2;
    Real lj12 = lj6 * lj6;
    Real lj12m6 = lj12 - lj6;
    Real scale = eps24 * r2inv * (lj12 + lj12m6);
    f[0] = d[0] * scale; f[1] = d[1] * scale; f[2] = d[2] * scale;
    V[0] = md[0] * f[0]; V[1] = md[1] * f[1]; V[2] = md[2] * f[2];
    u = eps24 * lj12m6 + shift6;
}

// charge(1)-charge(2) (VCP.cpp:227-277): f on site 1
template <typename Real>
__device__ __forceinline__ void cc_body(const Real* d, Real q1, Real q2, Real* f, Real& u) {
    Real r2 = dot3(d, d);
    Real r2inv = rcp_<Real>(r2);
    Real rinv = sqrt_<Real>(r2inv);
    u = q1 * q2 * rinv;
    Real fac = u * r2inv;
    f[0] = d[0] * fac; f[1] = d[1] * fac; f[2] = d[2] * fac;
}

// charge(1)-dipole(2) (VCP.cpp:279-347): d = r_charge - r_dipole; f on the
// charge, T = torque on the dipole, u = pair energy.
template <typename Real>
__device__ __forceinline__ void cd_body(const Real* d, Real q, const Real* e, Real p, Real* f, Real* T, Real& u) {
    Real r2 = dot3(d, d);
    Real r2inv = rcp_<Real>(r2);
    Real rinv = sqrt_<Real>(r2inv);
    Real r3inv = r2inv * rinv;
    Real re = dot3(d, e);
    Real qpr3 = q * p * r3inv;
    Real fac = r2inv * (Real)3 * re;
    for (int c = 0; c < 3; ++c) f[c] = qpr3 * (e[c] - d[c] * fac);
    u = -(qpr3 * re);
    T[0] = qpr3 * (e[1] * d[2] - e[2] * d[1]);
    T[1] = qpr3 * (e[2] * d[0] - e[0] * d[2]);
    T[2] = qpr3 * (e[0] * d[1] - e[1] * d[0]);
}

// dipole(1)-dipole(2) with reaction field (VCP.cpp:349-442); with T2ON also
// the torque on dipole 2 (VCP.cpp:435-441), from the shared terms
template <typename Real, bool T2ON = false>
__device__ __forceinline__ void dd_body(const Real* d, const Real* ei, Real pi, const Real* ej, Real pj, Real epsRF,
                                        Real* f, Real* T1, Real& u, Real& urf, Real* T2 = nullptr) {
    Real r2 = dot3(d, d);
    Real r2inv = rcp_<Real>(r2);
    Real rinv = sqrt_<Real>(r2inv);
    Real r2three_inv = (Real)3 * r2inv;
    Real p1p2 = pi * pj;
    Real rffac = p1p2 * epsRF;
    Real p1p2r3 = p1p2 * rinv * r2inv;
    Real p1p2threer5 = p1p2r3 * r2three_inv;
    Real e1e2 = dot3(ei, ej);
    Real re1 = dot3(d, ei), re2 = dot3(d, ej);
    Real re2threeperr2 = re2 * r2three_inv;
    Real re1re2perr2 = r2inv * re1 * re2;
    Real e1e2m5 = e1e2 - (Real)5 * re1re2perr2;
    for (int c = 0; c < 3; ++c) f[c] = p1p2threer5 * (d[c] * e1e2m5 + (ei[c] * re2 + ej[c] * re1));
    u = p1p2r3 * (e1e2 - (Real)3 * re1re2perr2);
    urf = rffac * e1e2;
    Real x12[3] = {ei[1] * ej[2] - ei[2] * ej[1], ei[2] * ej[0] - ei[0] * ej[2], ei[0] * ej[1] - ei[1] * ej[0]};
    Real exd[3] = {ei[1] * d[2] - ei[2] * d[1], ei[2] * d[0] - ei[0] * d[2], ei[0] * d[1] - ei[1] * d[0]};
    for (int c = 0; c < 3; ++c) T1[c] = p1p2r3 * (re2threeperr2 * exd[c] - x12[c]) + rffac * x12[c];
    if (T2ON) {
        Real re1threeperr2 = re1 * r2three_inv;
        Real exd2[3] = {ej[1] * d[2] - ej[2] * d[1], ej[2] * d[0] - ej[0] * d[2], ej[0] * d[1] - ej[1] * d[0]};
        for (int c = 0; c < 3; ++c) T2[c] = p1p2r3 * (re1threeperr2 * exd2[c] + x12[c]) - rffac * x12[c];
    }
}

// charge(1)-quadrupole(2) (VCP.cpp:444-524): f on the charge, T on the quadrupole
template <typename Real>
__device__ __forceinline__ void cq_body(const Real* d, Real q, const Real* ej, Real m, Real* f, Real* T, Real& u) {
    Real r2 = dot3(d, d);
    Real invdr2 = rcp_<Real>(r2);
    Real invdr = sqrt_<Real>(invdr2);
    Real qQ05 = (Real)0.5 * q * m;
    Real costj = dot3(ej, d) * invdr;
    Real qQinv4dr3 = qQ05 * invdr * invdr2;
    u = qQinv4dr3 * ((Real)3 * costj * costj - (Real)1);
    Real minus_partialRijInvdr = (Real)3 * u * invdr2;
    Real partialTjInvdr = (Real)6 * costj * qQinv4dr3 * invdr;
    Real fac = costj * partialTjInvdr * invdr + minus_partialRijInvdr;
    for (int c = 0; c < 3; ++c) f[c] = fac * d[c] - partialTjInvdr * ej[c];
    T[0] = partialTjInvdr * (ej[2] * d[1] - ej[1] * d[2]);
    T[1] = partialTjInvdr * (ej[0] * d[2] - ej[2] * d[0]);
    T[2] = partialTjInvdr * (ej[1] * d[0] - ej[0] * d[1]);
}

// dipole(1)-quadrupole(2) (VCP.cpp:526-648): f on the dipole, T1 on the
// dipole, T2 on the quadrupole
template <typename Real>
__device__ __forceinline__ void dq_body(const Real* d, const Real* ei, Real p, const Real* ej, Real m, Real* f,
                                        Real* T1, Real* T2, Real& u) {
    Real r2 = dot3(d, d);
    Real invdr2 = rcp_<Real>(r2);
    Real invdr = sqrt_<Real>(invdr2);
    Real myqfac = (Real)1.5 * p * m * invdr2 * invdr2;
    Real costi = dot3(ei, d) * invdr;
    Real costj = dot3(ej, d) * invdr;
    Real cos2tj = costj * costj;
    Real cosgij = dot3(ei, ej);
    Real _5c2m1 = (Real)5 * cos2tj - (Real)1;
    Real _2costj = (Real)2 * costj;
    u = myqfac * (_2costj * cosgij - costi * _5c2m1);
    Real myqfacXinvdr = myqfac * invdr;
    Real mpR = (Real)4 * u * invdr2;
    Real mpTi = myqfacXinvdr * _5c2m1;
    Real mpTj = myqfacXinvdr * (Real)2 * ((Real)5 * (costi * costj) - cosgij);
    Real pG = myqfac * _2costj;
    Real fac = mpR - (costi * mpTi + costj * mpTj) * invdr;
    for (int c = 0; c < 3; ++c) f[c] = fac * d[c] + (mpTi * ei[c] + mpTj * ej[c]);
    Real g[3] = {pG * (ei[1] * ej[2] - ei[2] * ej[1]), pG * (ei[2] * ej[0] - ei[0] * ej[2]),
                 pG * (ei[0] * ej[1] - ei[1] * ej[0])};
    Real a[3] = {ei[1] * d[2] - ei[2] * d[1], ei[2] * d[0] - ei[0] * d[2], ei[0] * d[1] - ei[1] * d[0]};
    Real b[3] = {ej[1] * d[2] - ej[2] * d[1], ej[2] * d[0] - ej[0] * d[2], ej[0] * d[1] - ej[1] * d[0]};
    for (int c = 0; c < 3; ++c) { T1[c] = mpTi * a[c] - g[c]; T2[c] = mpTj * b[c] + g[c]; }
}

// quadrupole(1)-quadrupole(2) (VCP.cpp:650-792)
template <typename Real>
__device__ __forceinline__ void qq_body(const Real* d, const Real* ei, Real mi, const Real* ej, Real mj, Real* f,
                                        Real* T1, Real* T2, Real& u) {
    Real r2 = dot3(d, d);
    Real invdr2 = rcp_<Real>(r2);
    Real invdr = sqrt_<Real>(invdr2);
    Real qfac = (Real)0.75 * invdr * (mi * mj) * (invdr2 * invdr2);
    Real costi = dot3(ei, d) * invdr, costj = dot3(ej, d) * invdr;
    Real c2i = costi * costi, c2j = costj * costj;
    Real cosgij = dot3(ei, ej);
    Real term = cosgij - (Real)5 * (costi * costj);
    Real up = ((Real)1 + (Real)2 * term * term) - ((Real)5 * (c2i + c2j) + (Real)15 * c2i * c2j);
    u = qfac * up;
    Real mpR = (Real)5 * u * invdr2;
    Real p1 = qfac * (Real)10 * invdr;
    Real p2 = (Real)2 * term;
    Real mpTi = p1 * (costi + (p2 * costj + (Real)3 * costi * c2j));
    Real mpTj = p1 * (costj + (p2 * costi + (Real)3 * costj * c2i));
    Real pG = qfac * (Real)4 * term;
    Real fac = mpR - (mpTi * costi + mpTj * costj) * invdr;
    for (int c = 0; c < 3; ++c) f[c] = fac * d[c] + (mpTi * ei[c] + mpTj * ej[c]);
    Real g[3] = {pG * (ei[1] * ej[2] - ei[2] * ej[1]), pG * (ei[2] * ej[0] - ei[0] * ej[2]),
                 pG * (ei[0] * ej[1] - ei[1] * ej[0])};
    Real a[3] = {ei[1] * d[2] - ei[2] * d[1], ei[2] * d[0] - ei[0] * d[2], ei[0] * d[1] - ei[1] * d[0]};
    Real b[3] = {ej[1] * d[2] - ej[2] * d[1], ej[2] * d[0] - ej[0] * d[2], ej[0] * d[1] - ej[1] * d[0]};
    for (int c = 0; c < 3; ++c) { T1[c] = mpTi * a[c] - g[c]; T2[c] = mpTj * b[c] + g[c]; }
}

// Dispatch one electrostatic site pair (a of the thread's molecule, b of the
// neighbour): d = r_a - r_b, md = centre distance.  Returns the kind index
// (1 C-C, 2 C-D, 3 D-D, 4 C-Q, 5 D-Q, 6 Q-Q); f, T are the force and
// multipole torque on a; V = md o f; u the pair energy; urf the reaction-
// field term (dipole-dipole only).
template <typename Real>
__device__ __forceinline__ int multipole_pair(int ka, int kb, const Real* d, const Real* md, Real pa, const Real* ea,
                                              Real pb, const Real* eb, Real epsRF, Real* f, Real* V, Real* T, Real& u,
                                              Real& urf) {
    int kind = 0;
    Real tmp[3];
    urf = (Real)0;
    T[0] = T[1] = T[2] = (Real)0;
    if (ka == SK_CHARGE && kb == SK_CHARGE) {
        cc_body<Real>(d, pa, pb, f, u);
        kind = 1;
    } else if (ka == SK_CHARGE && kb == SK_DIPOLE) {
        cd_body<Real>(d, pa, eb, pb, f, tmp, u);
        kind = 2;
    } else if (ka == SK_DIPOLE && kb == SK_CHARGE) {
        Real nd[3] = {-d[0], -d[1], -d[2]};
        cd_body<Real>(nd, pb, ea, pa, f, T, u);
        f[0] = -f[0]; f[1] = -f[1]; f[2] = -f[2];
        kind = 2;
    } else if (ka == SK_DIPOLE && kb == SK_DIPOLE) {
        dd_body<Real>(d, ea, pa, eb, pb, epsRF, f, T, u, urf);
        kind = 3;
    } else if (ka == SK_CHARGE && kb == SK_QUAD) {
        cq_body<Real>(d, pa, eb, pb, f, tmp, u);
        kind = 4;
    } else if (ka == SK_QUAD && kb == SK_CHARGE) {
        Real nd[3] = {-d[0], -d[1], -d[2]};
        cq_body<Real>(nd, pb, ea, pa, f, T, u);
        f[0] = -f[0]; f[1] = -f[1]; f[2] = -f[2];
        kind = 4;
    } else if (ka == SK_DIPOLE && kb == SK_QUAD) {
        dq_body<Real>(d, ea, pa, eb, pb, f, T, tmp, u);
        kind = 5;
    } else if (ka == SK_QUAD && kb == SK_DIPOLE) {
        Real nd[3] = {-d[0], -d[1], -d[2]};
        dq_body<Real>(nd, eb, pb, ea, pa, f, tmp, T, u);
        f[0] = -f[0]; f[1] = -f[1]; f[2] = -f[2];
        kind = 5;
    } else if (ka == SK_QUAD && kb == SK_QUAD) {
        qq_body<Real>(d, ea, pa, eb, pb, f, T, tmp, u);
        kind = 6;
    } else {
        f[0] = f[1] = f[2] = (Real)0;
        u = (Real)0;
    }
    V[0] = md[0] * f[0]; V[1] = md[1] * f[1]; V[2] = md[2] * f[2];
    return kind;
}

}  // namespace md
