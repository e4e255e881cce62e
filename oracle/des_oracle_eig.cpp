// TEST INFRASTRUCTURE -- 3x3 symmetric eigen-solver of the CPU oracle,
// restated from Kopp, "Numerical diagonalization of hermitian 3x3 matrices",
// arXiv physics/0610206 (the reference's vendored 3x3-C library:
// dsyevc3.c:31-81, dsytrd3.c:28-105, dsyevq3.c:29-135, dsyevh3.c:31-135).
// Built twice: strict IEEE (the order of operations the GPU follows) and with
// the flags 3x3-C/Makefile gives the reference (-O3 -ffast-math).
#include <cfloat>
#include <cmath>

namespace {

inline double sq(double x) { return x * x; }

void eig_cardano(const double A[3][3], double w[3])            // dsyevc3.c:31-81
{
    double de = A[0][1] * A[1][2];
    double dd = sq(A[0][1]);
    double ee = sq(A[1][2]);
    double ff = sq(A[0][2]);
    double m = A[0][0] + A[1][1] + A[2][2];
    double c1 = (A[0][0] * A[1][1] + A[0][0] * A[2][2] + A[1][1] * A[2][2]) - (dd + ee + ff);
    double c0 = A[2][2] * dd + A[0][0] * ee + A[1][1] * ff - A[0][0] * A[1][1] * A[2][2] -
                2.0 * A[0][2] * de;
    double p = sq(m) - 3.0 * c1;
    double q = m * (p - (3.0 / 2.0) * c1) - (27.0 / 2.0) * c0;
    double sqrt_p = std::sqrt(std::fabs(p));
    double phi = 27.0 * (0.25 * sq(c1) * (p - c1) + c0 * (q + 27.0 / 4.0 * c0));
    phi = (1.0 / 3.0) * std::atan2(std::sqrt(std::fabs(phi)), q);
    double c = sqrt_p * std::cos(phi);
    double s = (1.0 / 1.73205080756887729352744634151) * sqrt_p * std::sin(phi);
    w[1] = (1.0 / 3.0) * (m - c);
    w[2] = w[1] + s;
    w[0] = w[1] + c;
    w[1] -= s;
}

void householder3(const double A[3][3], double Q[3][3], double d[3], double e[2])   // dsytrd3.c
{
    double u[3], q[3];
    double omega, f, K, h, g;
    for (int i = 0; i < 3; i++) {
        Q[i][i] = 1.0;
        for (int j = 0; j < i; j++) Q[i][j] = Q[j][i] = 0.0;
    }
    h = sq(A[0][1]) + sq(A[0][2]);
    if (A[0][1] > 0)
        g = -std::sqrt(h);
    else
        g = std::sqrt(h);
    e[0] = g;
    f = g * A[0][1];
    u[1] = A[0][1] - g;
    u[2] = A[0][2];
    omega = h - f;
    if (omega > 0.0) {
        omega = 1.0 / omega;
        K = 0.0;
        for (int i = 1; i < 3; i++) {
            f = A[1][i] * u[1] + A[i][2] * u[2];
            q[i] = omega * f;
            K += u[i] * f;
        }
        K *= 0.5 * sq(omega);
        for (int i = 1; i < 3; i++) q[i] = q[i] - K * u[i];
        d[0] = A[0][0];
        d[1] = A[1][1] - 2.0 * q[1] * u[1];
        d[2] = A[2][2] - 2.0 * q[2] * u[2];
        for (int j = 1; j < 3; j++) {
            f = omega * u[j];
            for (int i = 1; i < 3; i++) Q[i][j] = Q[i][j] - f * u[i];
        }
        e[1] = A[1][2] - q[1] * u[2] - u[1] * q[2];
    } else {
        for (int i = 0; i < 3; i++) d[i] = A[i][i];
        e[1] = A[1][2];
    }
}

int eig_ql(const double A[3][3], double Q[3][3], double w[3])   // dsyevq3.c:29-135
{
    double e[3];
    double g, r, p, f, b, s, c, t;
    householder3(A, Q, w, e);
    for (int l = 0; l < 2; l++) {
        int nIter = 0;
        int m;
        while (1) {
            for (m = l; m <= 1; m++) {
                g = std::fabs(w[m]) + std::fabs(w[m + 1]);
                if (std::fabs(e[m]) + g == g) break;
            }
            if (m == l) break;
            if (nIter++ >= 30) return -1;
            g = (w[l + 1] - w[l]) / (e[l] + e[l]);
            r = std::sqrt(sq(g) + 1.0);
            if (g > 0)
                g = w[m] - w[l] + e[l] / (g + r);
            else
                g = w[m] - w[l] + e[l] / (g - r);
            s = c = 1.0;
            p = 0.0;
            for (int i = m - 1; i >= l; i--) {
                f = s * e[i];
                b = c * e[i];
                if (std::fabs(f) > std::fabs(g)) {
                    c = g / f;
                    r = std::sqrt(sq(c) + 1.0);
                    e[i + 1] = f * r;
                    c *= (s = 1.0 / r);
                } else {
                    s = f / g;
                    r = std::sqrt(sq(s) + 1.0);
                    e[i + 1] = g * r;
                    s *= (c = 1.0 / r);
                }
                g = w[i + 1] - p;
                r = (w[i] - g) * s + 2.0 * c * b;
                p = s * r;
                w[i + 1] = g + p;
                g = c * r - b;
                for (int k = 0; k < 3; k++) {
                    t = Q[k][i + 1];
                    Q[k][i + 1] = s * Q[k][i] + c * t;
                    Q[k][i] = c * Q[k][i] - s * t;
                }
            }
            w[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        }
    }
    return 0;
}

}  // namespace

extern "C" int dso_eig_hybrid(const double A[3][3], double Q[3][3], double w[3])   // dsyevh3.c:31-135
{
    double norm, error, t, u;
    eig_cardano(A, w);
    t = std::fabs(w[0]);
    if ((u = std::fabs(w[1])) > t) t = u;
    if ((u = std::fabs(w[2])) > t) t = u;
    if (t < 1.0)
        u = t;
    else
        u = sq(t);
    error = 256.0 * DBL_EPSILON * sq(u);
    Q[0][1] = A[0][1] * A[1][2] - A[0][2] * A[1][1];
    Q[1][1] = A[0][2] * A[0][1] - A[1][2] * A[0][0];
    Q[2][1] = sq(A[0][1]);
    Q[0][0] = Q[0][1] + A[0][2] * w[0];
    Q[1][0] = Q[1][1] + A[1][2] * w[0];
    Q[2][0] = (A[0][0] - w[0]) * (A[1][1] - w[0]) - Q[2][1];
    norm = sq(Q[0][0]) + sq(Q[1][0]) + sq(Q[2][0]);
    if (norm <= error) return eig_ql(A, Q, w) == 0 ? 1 : -1;
    norm = std::sqrt(1.0 / norm);
    for (int j = 0; j < 3; j++) Q[j][0] = Q[j][0] * norm;
    Q[0][1] = Q[0][1] + A[0][2] * w[1];
    Q[1][1] = Q[1][1] + A[1][2] * w[1];
    Q[2][1] = (A[0][0] - w[1]) * (A[1][1] - w[1]) - Q[2][1];
    norm = sq(Q[0][1]) + sq(Q[1][1]) + sq(Q[2][1]);
    if (norm <= error) return eig_ql(A, Q, w) == 0 ? 1 : -1;
    norm = std::sqrt(1.0 / norm);
    for (int j = 0; j < 3; j++) Q[j][1] = Q[j][1] * norm;
    Q[0][2] = Q[1][0] * Q[2][1] - Q[2][0] * Q[1][1];
    Q[1][2] = Q[2][0] * Q[0][1] - Q[0][0] * Q[2][1];
    Q[2][2] = Q[0][0] * Q[1][1] - Q[1][0] * Q[0][1];
    return 0;
}

