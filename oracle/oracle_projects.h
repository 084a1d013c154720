/* ORACLE (test infrastructure only).
 *
 * CPU restatement of the per-cell stencils and of the project hooks the
 * oracle runs.  Every expression keeps the operand order of the cited
 * reference code so that, compiled with -ffp-contract=off, the results agree
 * bit for bit with the reference's own headers (checked against the
 * reference build in oracle/_ref by tests/test_oracle_ref.py).
 *
 *   Laplacian<1..3>, Gradient<1..3> .... source/utils/sledgehamr_utils.h:60-188
 *   KreissOligerDissipation<2,3> ....... source/kernels.h:65-106
 *   AxionStrings ....................... projects/AxionStrings/kernels_rhs.h:21-135,
 *                                        kernels_tagging.h:16-131
 *   NextToMinimalExample ............... projects/NextToMinimalExample/
 *                                        NextToMinimalExample.h:11-43
 *   MinimalExample ..................... projects/MinimalExample/MinimalExample.h:10-39
 *   FirstOrderPhaseTransition .......... projects/FirstOrderPhaseTransition/
 *                                        kernels_rhs.h:20-109, kernels_tagging.h:13-45
 *   AxionStringsLapN (N = 1, 2, 3) ..... the lattice-order variant of the axion
 *                                        string equations used by the 128^3 and
 *                                        ensemble workloads: NextToMinimalExample's
 *                                        Rhs with Laplacian order N and the constant
 *                                        0.56233 replaced by params[1].
 */
#ifndef SH_ORACLE_PROJECTS_H_
#define SH_ORACLE_PROJECTS_H_

#include "oracle_core.h"

namespace orc {

using S4 = A4<const double>;
using R4 = A4<double>;

template <int O>
inline double lap(const S4 &s, int i, int j, int k, int c, double dx2);
template <>
inline double lap<1>(const S4 &s, int i, int j, int k, int c, double dx2) {
    return (s(i + 1, j, k, c) + s(i - 1, j, k, c) + s(i, j + 1, k, c) + s(i, j - 1, k, c) +
            s(i, j, k + 1, c) + s(i, j, k - 1, c) - 6. * s(i, j, k, c)) /
           dx2;
}
template <>
inline double lap<2>(const S4 &s, int i, int j, int k, int c, double dx2) {
    return (-(s(i + 2, j, k, c) + s(i - 2, j, k, c) + s(i, j + 2, k, c) + s(i, j - 2, k, c) +
              s(i, j, k + 2, c) + s(i, j, k - 2, c)) +
            16. * (s(i + 1, j, k, c) + s(i - 1, j, k, c) + s(i, j + 1, k, c) + s(i, j - 1, k, c) +
                   s(i, j, k + 1, c) + s(i, j, k - 1, c)) -
            90. * s(i, j, k, c)) /
           (12. * dx2);
}
template <>
inline double lap<3>(const S4 &s, int i, int j, int k, int c, double dx2) {
    return (2. * (s(i + 3, j, k, c) + s(i - 3, j, k, c) + s(i, j + 3, k, c) + s(i, j - 3, k, c) +
                  s(i, j, k + 3, c) + s(i, j, k - 3, c)) -
            27. * (s(i + 2, j, k, c) + s(i - 2, j, k, c) + s(i, j + 2, k, c) + s(i, j - 2, k, c) +
                   s(i, j, k + 2, c) + s(i, j, k - 2, c)) +
            270. * (s(i + 1, j, k, c) + s(i - 1, j, k, c) + s(i, j + 1, k, c) + s(i, j - 1, k, c) +
                    s(i, j, k + 1, c) + s(i, j, k - 1, c)) -
            1470. * s(i, j, k, c)) /
           (180. * dx2);
}

/* value at offset d along axis ax (0 = x, 1 = y, 2 = z) */
inline double at(const S4 &s, int i, int j, int k, int c, int ax, int d) {
    return ax == 0 ? s(i + d, j, k, c) : (ax == 1 ? s(i, j + d, k, c) : s(i, j, k + d, c));
}

template <int O>
inline double grad(const S4 &s, int i, int j, int k, int c, double dx, int ax);
template <>
inline double grad<1>(const S4 &s, int i, int j, int k, int c, double dx, int ax) {
    return (at(s, i, j, k, c, ax, 1) - at(s, i, j, k, c, ax, -1)) / (2. * dx);
}
template <>
inline double grad<2>(const S4 &s, int i, int j, int k, int c, double dx, int ax) {
    return (-at(s, i, j, k, c, ax, 2) + 8. * at(s, i, j, k, c, ax, 1) + at(s, i, j, k, c, ax, -2) -
            8. * at(s, i, j, k, c, ax, -1)) /
           (12. * dx);
}
template <>
inline double grad<3>(const S4 &s, int i, int j, int k, int c, double dx, int ax) {
    return (+at(s, i, j, k, c, ax, 3) - at(s, i, j, k, c, ax, -3) - 9. * at(s, i, j, k, c, ax, 2) +
            9. * at(s, i, j, k, c, ax, -2) + 45. * at(s, i, j, k, c, ax, 1) -
            45. * at(s, i, j, k, c, ax, -1)) /
           (60. * dx);
}

inline double ko_dissipation(int order, const S4 &s, int i, int j, int k, int c, double dx,
                             double strength) {
    if (order == 2) {
        double d[3];
        for (int ax = 0; ax < 3; ++ax)
            d[ax] = at(s, i, j, k, c, ax, 2) - 4. * at(s, i, j, k, c, ax, 1) +
                    at(s, i, j, k, c, ax, -2) - 4. * at(s, i, j, k, c, ax, -1) +
                    6. * s(i, j, k, c);
        return -strength * (d[0] + d[1] + d[2]) / 16. / dx;
    }
    double d[3];
    for (int ax = 0; ax < 3; ++ax)
        d[ax] = at(s, i, j, k, c, ax, 3) - 6. * at(s, i, j, k, c, ax, 2) +
                15. * at(s, i, j, k, c, ax, 1) + at(s, i, j, k, c, ax, -3) -
                6. * at(s, i, j, k, c, ax, -2) + 15. * at(s, i, j, k, c, ax, -1) -
                20. * s(i, j, k, c);
    return strength * (d[0] + d[1] + d[2]) / 64. / dx;
}

/* ---- axion-string plaquette winding (kernels_tagging.h:16-108) ---------- */
inline int zero_xing(double a1, double a2, double b1, double b2) {
    if (a2 * b2 >= 0) return 0;
    if (a2 * b1 - a1 * b2 > 0) return 1;
    return -1;
}
/* Winding around the plaquette spanned by axes p and q at corner (i,j,k);
 * corners visited (0,0) -> (1,0) -> (1,1) -> (0,1) -> (0,0). */
inline int winding(const S4 &s, int i, int j, int k, int p, int q, int c1, int c2) {
    auto off = [&](int dp, int dq, int &ii, int &jj, int &kk) {
        ii = i; jj = j; kk = k;
        (p == 0 ? ii : (p == 1 ? jj : kk)) += dp;
        (q == 0 ? ii : (q == 1 ? jj : kk)) += dq;
    };
    const int cp[5] = {0, 1, 1, 0, 0}, cq[5] = {0, 0, 1, 1, 0};
    int w = 0;
    for (int e = 0; e < 4; ++e) {
        int i0, j0, k0, i1, j1, k1;
        off(cp[e], cq[e], i0, j0, k0);
        off(cp[e + 1], cq[e + 1], i1, j1, k1);
        w += zero_xing(s(i0, j0, k0, c1), s(i0, j0, k0, c2), s(i1, j1, k1, c1), s(i1, j1, k1, c2));
    }
    return w;
}
inline bool string_tag(const S4 &s, int i, int j, int k, int c1, int c2) {
    if (winding(s, i, j, k, 0, 1, c1, c2) != 0) return true; /* WindingAxis1: x-y */
    if (winding(s, i, j, k, 0, 2, c1, c2) != 0) return true; /* WindingAxis2: x-z */
    if (winding(s, i, j, k, 1, 2, c1, c2) != 0) return true; /* WindingAxis3: y-z */
    return false;
}

/* ---- project policies ----------------------------------------------------- */
struct NoGw {
    static void gw_rhs(const R4 &, const S4 &, int, int, int, int, double, double, double,
                       const double *) {}
    static void gw_backreaction(const R4 &, const S4 &, int, int, int, int, double, double,
                                double, const double *, const double *) {}
};

/* Complex scalar (Psi1, Psi2, Pi1, Pi2) with the axion-string potential. */
template <int Order, int Variant>
struct AxionFamily : NoGw {
    /* Variant 0: AxionStrings (+0.56233, winding tags, dt-scaled momentum
     *            truncation errors);
     * 1: NextToMinimalExample (potential x params[0], default tag hooks);
     * 2: AxionStringsLapN (potential x params[0] with constant params[1],
     *    AxionStrings tag hooks);
     * 3: MinimalExample (+0.56233, default tag hooks). */
    static constexpr bool kStringTags = (Variant == 0 || Variant == 2);
    static constexpr int NScalars = 4, NFields = 2;
    static constexpr int Psi1 = 0, Psi2 = 1, Pi1 = 2, Pi2 = 3;
    static void rhs(const R4 &rhs, const S4 &state, int i, int j, int k, int lev, double time,
                    double dt, double dx, const double *params) {
        double P1 = state(i, j, k, Psi1), P2 = state(i, j, k, Psi2);
        double Q1 = state(i, j, k, Pi1), Q2 = state(i, j, k, Pi2);
        double eta = time;
        double l1 = lap<Order>(state, i, j, k, Psi1, dx * dx);
        double l2 = lap<Order>(state, i, j, k, Psi2, dx * dx);
        double potential;
        if (Variant == 0 || Variant == 3) {
            potential = eta * eta * (P1 * P1 + P2 * P2 - 1.) + 0.56233;
        } else if (Variant == 1) {
            potential = eta * eta * (P1 * P1 + P2 * P2 - 1.) + 0.56233;
            potential *= params[0];
        } else {
            potential = eta * eta * (P1 * P1 + P2 * P2 - 1.) + params[1];
            potential *= params[0];
        }
        rhs(i, j, k, Psi1) = Q1;
        rhs(i, j, k, Psi2) = Q2;
        rhs(i, j, k, Pi1) = -Q1 * 2. / eta + l1 - P1 * potential;
        rhs(i, j, k, Pi2) = -Q2 * 2. / eta + l2 - P2 * potential;
    }
    static bool tag(const S4 &s, int i, int j, int k, int, double, double, double,
                    const double *) {
        return kStringTags ? string_tag(s, i, j, k, Psi1, Psi2) : false;
    }
    /* AxionStrings modifies Pi1, Pi2 and du_* by dt (kernels_tagging.h:115-131);
     * MinimalExample and NextToMinimalExample keep the default. */
    static double te_modifier(int n, const S4 &, int, int, int, int, double, double dt, double,
                              double te, const double *) {
        if (!kStringTags) return te;
        bool by_dt = (n == Pi1 || n == Pi2 || (n >= 4 + 6 && n < 4 + 12));
        return by_dt ? te * dt : te;
    }
    static double ko(int order, const S4 &s, int i, int j, int k, int n, double dx, double str) {
        return ko_dissipation(order, s, i, j, k, n, dx, str);
    }
};

/* AxionStrings: Rhs as Variant 0 with order 2, and its GW source hook that
 * writes the u_* slots twice and never the du_* slots (kernels_rhs.h:110-134). */
struct AxionStrings : AxionFamily<2, 0> {
    static void gw_rhs(const R4 &rhs, const S4 &state, int i, int j, int k, int lev, double time,
                       double dt, double dx, const double *params) {
        const int u0 = 4, du0 = 10; /* u_xx..u_yz, du_xx..du_yz */
        double du[6];
        for (int q = 0; q < 6; ++q) du[q] = state(i, j, k, du0 + q);
        double eta = time;
        double dx2 = dx * dx;
        double lu[6];
        for (int q = 0; q < 6; ++q) lu[q] = lap<2>(state, i, j, k, u0 + q, dx2);
        double g1[3], g2[3];
        for (int ax = 0; ax < 3; ++ax) {
            g1[ax] = grad<2>(state, i, j, k, 0, dx, ax);
            g2[ax] = grad<2>(state, i, j, k, 1, dx, ax);
        }
        for (int q = 0; q < 6; ++q) rhs(i, j, k, u0 + q) = du[q];
        /* order of the tensor slots: xx, yy, zz, xy, xz, yz */
        const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
        for (int q = 0; q < 6; ++q)
            rhs(i, j, k, u0 + q) = -du[q] * 2. / eta + lu[q] + g1[pa[q]] * g1[pb[q]] +
                                   g2[pa[q]] * g2[pb[q]];
    }
};
using MinimalExample = AxionFamily<2, 3>;
using NextToMinimalExample = AxionFamily<2, 1>;
template <int O>
using AxionStringsLap = AxionFamily<O, 2>;

/* FirstOrderPhaseTransition: real scalar (Phi, dPhi) + GW tensor. */
struct FirstOrderPhaseTransition {
    static constexpr int NScalars = 2, NFields = 1;
    static constexpr int Phi = 0, dPhi = 1;
    static void rhs(const R4 &rhs, const S4 &state, int i, int j, int k, int lev, double time,
                    double dt, double dx, const double *params) {
        int potential_type = static_cast<int>(params[0]);
        double quadratic = params[1], cubic = params[2], quartic = params[3];
        double vbar = params[4], vareps = params[5], phiesc = params[6];
        double P = state(i, j, k, Phi);
        double potential = 0;
        if (potential_type == 0) {
            potential = quadratic * P + cubic * P * P + quartic * P * P * P;
        } else if (potential_type == 1) {
            double cond = P < phiesc;
            potential = cond * (quadratic * P + cubic * P * P + quartic * P * P * P) -
                        (1 - cond) * vareps * vareps * (P - vbar);
        }
        double l = lap<2>(state, i, j, k, Phi, dx * dx);
        rhs(i, j, k, Phi) = state(i, j, k, dPhi);
        rhs(i, j, k, dPhi) = l + potential;
    }
    static void gw_rhs(const R4 &rhs, const S4 &state, int i, int j, int k, int lev, double time,
                       double dt, double dx, const double *params) {
        const int u0 = 2, du0 = 8;
        double dx2 = dx * dx;
        double lu[6];
        for (int q = 0; q < 6; ++q) lu[q] = lap<2>(state, i, j, k, u0 + q, dx2);
        double g[3];
        for (int ax = 0; ax < 3; ++ax) g[ax] = grad<2>(state, i, j, k, Phi, dx, ax);
        double C = 1;
        for (int q = 0; q < 6; ++q) rhs(i, j, k, u0 + q) = state(i, j, k, du0 + q);
        const int pa[6] = {0, 1, 2, 0, 0, 1}, pb[6] = {0, 1, 2, 1, 2, 2};
        for (int q = 0; q < 6; ++q) rhs(i, j, k, du0 + q) = (lu[q] + g[pa[q]] * g[pb[q]]) * C;
    }
    static void gw_backreaction(const R4 &, const S4 &, int, int, int, int, double, double,
                                double, const double *, const double *) {}
    static bool tag(const S4 &, int, int, int, int, double, double, double, const double *) {
        return false;
    }
    /* kernels_tagging.h:13-45: te / max|comp|, times dt for momenta. */
    static double te_modifier(int n, const S4 &, int, int, int, int, double, double dt, double,
                              double te, const double *params) {
        bool by_dt = (n == dPhi || (n >= 8 && n < 14));
        return by_dt ? te * dt / params[n] : te / params[n];
    }
    static double ko(int order, const S4 &s, int i, int j, int k, int n, double dx, double str) {
        return ko_dissipation(order, s, i, j, k, n, dx, str);
    }
};

} // namespace orc

#endif // SH_ORACLE_PROJECTS_H_
