// dg_basis.cpp -- see dg_basis.hpp.  Independent FP64 implementation (Gauss
// rules by Newton iteration, inverses by Gauss-Jordan); results agree with
// the reference's PETSc/SLEPc-based construction to round-off.
#include "dg_basis.hpp"

#include <cmath>
#include <cstdio>

namespace dgb {

namespace {

typedef std::vector<double> vec;

// Orthonormal Jacobi polynomial P_n^{(a,b)} at x (three-term recurrence).
double jacobi(double x, double a, double b, int n) {
    double g0 = std::pow(2.0, a + b + 1) / (a + b + 1) * std::tgamma(a + 1) * std::tgamma(b + 1) / std::tgamma(a + b + 1);
    double p0 = 1.0 / std::sqrt(g0);
    if (n == 0) return p0;
    double g1 = (a + 1) * (b + 1) / (a + b + 3) * g0;
    double p1 = ((a + b + 2) * x / 2 + (a - b) / 2) / std::sqrt(g1);
    if (n == 1) return p1;
    double aold = 2 / (2 + a + b) * std::sqrt((a + 1) * (b + 1) / (a + b + 3));
    for (int i = 1; i < n; i++) {
        double h1 = 2.0 * i + a + b;
        double anew = 2 / (h1 + 2) * std::sqrt((i + 1) * (i + 1 + a + b) * (i + 1 + a) * (i + 1 + b) / (h1 + 1) / (h1 + 3));
        double bnew = -(a * a - b * b) / h1 / (h1 + 2);
        double p2 = ((x - bnew) * p1 - aold * p0) / anew;
        p0 = p1;
        p1 = p2;
        aold = anew;
    }
    return p1;
}

double djacobi(double x, double a, double b, int n) {
    if (n == 0) return 0.0;
    return std::sqrt(n * (n + a + b + 1)) * jacobi(x, a + 1, b + 1, n - 1);
}

// Classical Legendre P_n and P_n' (unnormalised) at x.
void legendre(int n, double x, double& p, double& dp) {
    double p0 = 1, p1 = x;
    if (n == 0) { p = 1; dp = 0; return; }
    for (int k = 2; k <= n; k++) {
        double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
    }
    p = p1;
    dp = n * (x * p1 - p0) / (x * x - 1);
}

// Gauss-Legendre rule with n points, ascending, symmetrised weights.
void gauss_legendre(int n, vec& x, vec& w) {
    const double pi = 3.14159265358979323846;
    x.assign(n, 0);
    w.assign(n, 0);
    for (int i = 0; i < n; i++) {
        double z = -std::cos(pi * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; it++) {
            double p, dp;
            legendre(n, z, p, dp);
            double dz = p / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p, dp;
        legendre(n, z, p, dp);
        x[i] = z;
        w[i] = 2.0 / ((1 - z * z) * dp * dp);
    }
    for (int i = 0; i < n / 2; i++) {  // exact symmetry
        double xm = 0.5 * (x[n - 1 - i] - x[i]);
        x[i] = -xm;
        x[n - 1 - i] = xm;
        double wm = 0.5 * (w[i] + w[n - 1 - i]);
        w[i] = w[n - 1 - i] = wm;
    }
    if (n % 2) x[n / 2] = 0.0;
}

// Gauss-Lobatto-Legendre nodes (N+1 points): -1, roots of P_N', 1.
vec gauss_lobatto(int N) {
    const double pi = 3.14159265358979323846;
    vec x(N + 1);
    x[0] = -1;
    x[N] = 1;
    for (int i = 1; i < N; i++) {
        double z = -std::cos(pi * i / N);
        for (int it = 0; it < 100; it++) {
            double p, dp;
            legendre(N, z, p, dp);
            // q = P_N', q' = (2 z P_N' - N(N+1) P_N) / (1 - z^2)
            double ddp = (2 * z * dp - N * (N + 1) * p) / (1 - z * z);
            double dz = dp / ddp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[i] = z;
    }
    for (int i = 0; i < (N + 1) / 2; i++) {
        double xm = 0.5 * (x[N - i] - x[i]);
        x[i] = -xm;
        x[N - i] = xm;
    }
    if (N % 2 == 0) x[N / 2] = 0.0;
    return x;
}

bool invert(const vec& A, int n, vec& X) {
    vec M(A);
    X.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; i++) X[(size_t)i * n + i] = 1.0;
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int i = c + 1; i < n; i++)
            if (std::fabs(M[(size_t)i * n + c]) > std::fabs(M[(size_t)p * n + c])) p = i;
        if (M[(size_t)p * n + c] == 0.0) return false;
        if (p != c)
            for (int j = 0; j < n; j++) {
                std::swap(M[(size_t)p * n + j], M[(size_t)c * n + j]);
                std::swap(X[(size_t)p * n + j], X[(size_t)c * n + j]);
            }
        double inv = 1.0 / M[(size_t)c * n + c];
        for (int j = 0; j < n; j++) {
            M[(size_t)c * n + j] *= inv;
            X[(size_t)c * n + j] *= inv;
        }
        for (int i = 0; i < n; i++) {
            if (i == c) continue;
            double f = M[(size_t)i * n + c];
            if (f == 0.0) continue;
            for (int j = 0; j < n; j++) {
                M[(size_t)i * n + j] -= f * M[(size_t)c * n + j];
                X[(size_t)i * n + j] -= f * X[(size_t)c * n + j];
            }
        }
    }
    return true;
}

vec matmul(const vec& A, const vec& B, int m, int k, int n) {
    vec C((size_t)m * n, 0.0);
    for (int i = 0; i < m; i++)
        for (int l = 0; l < k; l++) {
            double a = A[(size_t)i * k + l];
            for (int j = 0; j < n; j++) C[(size_t)i * n + j] += a * B[(size_t)l * n + j];
        }
    return C;
}

// Dubiner basis value and gradient at (r, s); modes ordered (i, j), j fastest.
void simplex_basis(int N, double r, double s, double* phi, double* dr, double* ds) {
    double a = (s != 1.0) ? 2 * (1 + r) / (1 - s) - 1 : -1.0;
    double b = s;
    int sk = 0;
    for (int i = 0; i <= N; i++)
        for (int j = 0; j <= N - i; j++) {
            double fa = jacobi(a, 0, 0, i), gb = jacobi(b, 2 * i + 1, 0, j);
            double dfa = djacobi(a, 0, 0, i), dgb = djacobi(b, 2 * i + 1, 0, j);
            double nrm = std::pow(2.0, i + 0.5);
            if (phi) phi[sk] = std::sqrt(2.0) * fa * gb * std::pow(1 - b, i);
            double om = 0.5 * (1 - b);
            double omi1 = (i > 0) ? std::pow(om, i - 1) : 1.0;
            double dmr = dfa * gb * omi1;
            double dms = dfa * gb * 0.5 * (1 + a) * omi1;
            double t = dgb * std::pow(om, i);
            if (i > 0) t -= 0.5 * i * gb * std::pow(om, i - 1);
            dms += fa * t;
            if (dr) dr[sk] = dmr * nrm;
            if (ds) ds[sk] = dms * nrm;
            sk++;
        }
}

// warp function of the warp & blend construction (1D LGL vs equispaced)
double warp1d(int N, double x, const vec& lgl) {
    // Lagrange interpolant through equispaced nodes of (lgl - equispaced)
    double w = 0;
    for (int i = 0; i <= N; i++) {
        double xi = -1.0 + 2.0 * i / N;
        double l = 1;
        for (int j = 0; j <= N; j++)
            if (j != i) l *= (x - (-1.0 + 2.0 * j / N)) / (xi - (-1.0 + 2.0 * j / N));
        w += l * (lgl[i] - xi);
    }
    if (std::fabs(x) < 1.0 - 1e-10) w /= (1 - x * x);
    else w = 0.0;  // the reference zeroes the warp at the interval ends
    return w;
}

}  // namespace

int cubature_points_for_order(int N) {
    static const int tab[8] = {0, 12, 19, 36, 54, 73, 93, 118};
    return (N >= 1 && N <= 7) ? tab[N] : 0;
}

std::string build_ref_ops(int N, const double* cub, int Ng, RefOps& o) {
    if (N < 1 || N > 7) return "order must be in 1..7";
    if (!cub || Ng <= 0) return "cubature rule missing";
    o.N = N;
    o.Np = (N + 1) * (N + 2) / 2;
    o.Nfp = N + 1;
    o.Nfq = N + 2;
    o.Ng = Ng;
    int Np = o.Np, Nfp = o.Nfp, Nfq = o.Nfq;

    // warp & blend nodes
    static const double alpopt[15] = {0.0000, 0.0000, 1.4152, 0.1001, 0.2751, 0.9800, 1.0999, 1.2832,
                                      1.3648, 1.4773, 1.4959, 1.5743, 1.5770, 1.6223, 1.6258};
    double alpha = alpopt[N - 1];
    vec lgl = gauss_lobatto(N);
    o.r.assign(Np, 0);
    o.s.assign(Np, 0);
    const double pi = 3.14159265358979323846;
    int sk = 0;
    for (int n = 1; n <= N + 1; n++)
        for (int m = 1; m <= N + 2 - n; m++) {
            double L1 = (double)(n - 1) / N, L3 = (double)(m - 1) / N, L2 = 1.0 - L1 - L3;
            double X = L3 - L2, Y = (2 * L1 - L2 - L3) / std::sqrt(3.0);
            double w1 = 4 * L2 * L3 * warp1d(N, L3 - L2, lgl) * (1 + (alpha * L1) * (alpha * L1));
            double w2 = 4 * L1 * L3 * warp1d(N, L1 - L3, lgl) * (1 + (alpha * L2) * (alpha * L2));
            double w3 = 4 * L1 * L2 * warp1d(N, L2 - L1, lgl) * (1 + (alpha * L3) * (alpha * L3));
            X += w1 + std::cos(2 * pi / 3) * w2 + std::cos(4 * pi / 3) * w3;
            Y += std::sin(2 * pi / 3) * w2 + std::sin(4 * pi / 3) * w3;
            double l1 = (std::sqrt(3.0) * Y + 1.0) / 3.0;
            double l2 = (-3.0 * X - std::sqrt(3.0) * Y + 2.0) / 6.0;
            double l3 = (3.0 * X - std::sqrt(3.0) * Y + 2.0) / 6.0;
            o.r[sk] = l3 - l2 - l1;
            o.s[sk] = l1 - l2 - l3;
            sk++;
        }
    // face node ids (face direction), as faceToCellIndex[f][0]
    o.fnode.assign(3 * Nfp, 0);
    for (int i = 0; i < Nfp; i++) o.fnode[i] = i;
    o.fnode[Nfp] = N;
    o.fnode[2 * Nfp] = Np - 1;
    for (int i = 1; i < Nfp; i++) {
        o.fnode[Nfp + i] = o.fnode[Nfp + i - 1] + (Nfp - i);
        o.fnode[2 * Nfp + i] = o.fnode[2 * Nfp + i - 1] - i - 1;
    }
    // ring order
    o.ring.clear();
    std::vector<char> onb(Np, 0);
    for (int f = 0; f < 3; f++)
        for (int j = 0; j < N; j++) {
            o.ring.push_back(o.fnode[f * Nfp + j]);
            onb[o.fnode[f * Nfp + j]] = 1;
        }
    for (int i = 0; i < Np; i++)
        if (!onb[i]) o.ring.push_back(i);
    if ((int)o.ring.size() != Np) return "ring construction failed";

    // V, Vr, Vs at nodes
    o.V.assign((size_t)Np * Np, 0);
    vec Vr((size_t)Np * Np), Vs((size_t)Np * Np);
    for (int i = 0; i < Np; i++)
        simplex_basis(N, o.r[i], o.s[i], &o.V[(size_t)i * Np], &Vr[(size_t)i * Np], &Vs[(size_t)i * Np]);
    if (!invert(o.V, Np, o.invV)) return "singular Vandermonde";
    o.Dr = matmul(Vr, o.invV, Np, Np, Np);
    o.Ds = matmul(Vs, o.invV, Np, Np, Np);

    // cubature
    o.gr.resize(Ng);
    o.gs.resize(Ng);
    o.gw.resize(Ng);
    for (int g = 0; g < Ng; g++) { o.gr[g] = cub[3 * g]; o.gs[g] = cub[3 * g + 1]; o.gw[g] = cub[3 * g + 2]; }
    vec Bg((size_t)Ng * Np), Bgr((size_t)Ng * Np), Bgs((size_t)Ng * Np);
    for (int g = 0; g < Ng; g++)
        simplex_basis(N, o.gr[g], o.gs[g], &Bg[(size_t)g * Np], &Bgr[(size_t)g * Np], &Bgs[(size_t)g * Np]);
    o.Vg = matmul(Bg, o.invV, Ng, Np, Np);
    o.Drg = matmul(Bgr, o.invV, Ng, Np, Np);
    o.Dsg = matmul(Bgs, o.invV, Ng, Np, Np);

    // face Gauss rule (N+2 points) and face interpolation from the LGL face nodes
    gauss_legendre(Nfq, o.fq, o.fw);
    vec V1((size_t)Nfp * Nfp), Vq((size_t)Nfq * Nfp), invV1;
    for (int i = 0; i < Nfp; i++)
        for (int j = 0; j < Nfp; j++) V1[(size_t)i * Nfp + j] = jacobi(lgl[i], 0, 0, j);
    for (int i = 0; i < Nfq; i++)
        for (int j = 0; j < Nfp; j++) Vq[(size_t)i * Nfp + j] = jacobi(o.fq[i], 0, 0, j);
    if (!invert(V1, Nfp, invV1)) return "singular 1D Vandermonde";
    o.If = matmul(Vq, invV1, Nfq, Nfp, Nfp);

    // reference mass matrix by the cubature (as physicalCellElement::initMassMatrix, J = 1)
    o.Mref.assign((size_t)Np * Np, 0.0);
    for (int g = 0; g < Ng; g++)
        for (int i = 0; i < Np; i++)
            for (int j = 0; j < Np; j++) o.Mref[(size_t)i * Np + j] += o.Vg[(size_t)g * Np + i] * o.Vg[(size_t)g * Np + j] * o.gw[g];
    if (!invert(o.Mref, Np, o.Minv)) return "singular mass matrix";

    // fused operators (reference order first)
    vec Sr((size_t)Np * Ng, 0.0), Ss((size_t)Np * Ng, 0.0);
    for (int i = 0; i < Np; i++)
        for (int g = 0; g < Ng; g++) {
            double ar = 0, as = 0;
            for (int j = 0; j < Np; j++) {
                ar += o.Minv[(size_t)i * Np + j] * o.Drg[(size_t)g * Np + j];
                as += o.Minv[(size_t)i * Np + j] * o.Dsg[(size_t)g * Np + j];
            }
            Sr[(size_t)i * Ng + g] = ar * o.gw[g];
            Ss[(size_t)i * Ng + g] = as * o.gw[g];
        }
    vec Lift((size_t)Np * 3 * Nfq, 0.0);
    for (int i = 0; i < Np; i++)
        for (int f = 0; f < 3; f++)
            for (int q = 0; q < Nfq; q++) {
                double a = 0;
                for (int j = 0; j < Nfp; j++) a += o.Minv[(size_t)i * Np + o.fnode[f * Nfp + j]] * o.If[(size_t)q * Nfp + j];
                Lift[(size_t)i * 3 * Nfq + f * Nfq + q] = a * o.fw[q];
            }
    // permute to ring order
    o.dVg.assign((size_t)Ng * Np, 0);
    o.dSr.assign((size_t)Np * Ng, 0);
    o.dSs.assign((size_t)Np * Ng, 0);
    o.dLift.assign((size_t)Np * 3 * Nfq, 0);
    for (int p = 0; p < Np; p++) {
        int ref = o.ring[p];
        for (int g = 0; g < Ng; g++) {
            o.dVg[(size_t)g * Np + p] = o.Vg[(size_t)g * Np + ref];
            o.dSr[(size_t)p * Ng + g] = Sr[(size_t)ref * Ng + g];
            o.dSs[(size_t)p * Ng + g] = Ss[(size_t)ref * Ng + g];
        }
        for (int c = 0; c < 3 * Nfq; c++) o.dLift[(size_t)p * 3 * Nfq + c] = Lift[(size_t)ref * 3 * Nfq + c];
    }
    return "";
}

}  // namespace dgb
