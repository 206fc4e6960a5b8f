// mg.cu -- multilevel coarse-space correction of the SIPG PCG (see mg.hpp):
// host construction of the levels and the device V-cycle.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "euler_flux.cuh"
#include "mg.hpp"
#include "pcg_reduce.cuh"

namespace dgk {

namespace {

constexpr double kOmega = 0.6;  // weighted-Jacobi factor of the smoother
constexpr int kCoarsest = 500;  // largest operator solved by its dense inverse

// sums duplicate (i, j) triplets into CSR
void to_csr(int n, std::vector<long long>& key, std::vector<double>& v, MgBuild::Level& L) {
    std::vector<size_t> ord(key.size());
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return key[a] < key[b]; });
    L.n = n;
    L.rowptr.assign(n + 1, 0);
    L.col.clear();
    L.val.clear();
    long long last = -1;
    for (size_t q : ord) {
        if (key[q] != last) {
            L.col.push_back((int)(key[q] % n));
            L.val.push_back(v[q]);
            L.rowptr[key[q] / n + 1]++;
            last = key[q];
        } else {
            L.val.back() += v[q];
        }
    }
    for (int i = 0; i < n; i++) L.rowptr[i + 1] += L.rowptr[i];
}

void jacobi_of(MgBuild::Level& L) {
    L.dinv.assign(L.n, 0.0);
    for (int i = 0; i < L.n; i++)
        for (int q = L.rowptr[i]; q < L.rowptr[i + 1]; q++)
            if (L.col[q] == i) L.dinv[i] = kOmega / L.val[q];
}

// greedy aggregation on the matrix graph: each unassigned unknown opens an
// aggregate with its unassigned neighbours
int aggregate(const MgBuild::Level& L, std::vector<int>& agg) {
    agg.assign(L.n, -1);
    int na = 0;
    for (int i = 0; i < L.n; i++) {
        if (agg[i] >= 0) continue;
        agg[i] = na;
        for (int q = L.rowptr[i]; q < L.rowptr[i + 1]; q++)
            if (agg[L.col[q]] < 0) agg[L.col[q]] = na;
        na++;
    }
    return na;
}

// dense inverse of an SPD matrix by Cholesky; false if not positive definite
bool spd_inverse(int n, std::vector<double>& A) {
    std::vector<double> Lm(A);
    for (int j = 0; j < n; j++) {
        double d = Lm[(size_t)j * n + j];
        for (int k = 0; k < j; k++) d -= Lm[(size_t)j * n + k] * Lm[(size_t)j * n + k];
        if (!(d > 0)) return false;
        d = std::sqrt(d);
        Lm[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; i++) {
            double s = Lm[(size_t)i * n + j];
            for (int k = 0; k < j; k++) s -= Lm[(size_t)i * n + k] * Lm[(size_t)j * n + k];
            Lm[(size_t)i * n + j] = s / d;
        }
    }
    // inverse column by column: L y = e_c, L^T x = y
    std::vector<double> y(n);
    for (int c = 0; c < n; c++) {
        for (int i = 0; i < n; i++) {
            double s = (i == c) ? 1.0 : 0.0;
            for (int k = 0; k < i; k++) s -= Lm[(size_t)i * n + k] * y[k];
            y[i] = s / Lm[(size_t)i * n + i];
        }
        for (int i = n - 1; i >= 0; i--) {
            double s = y[i];
            for (int k = i + 1; k < n; k++) s -= Lm[(size_t)k * n + i] * A[(size_t)k * n + c];
            A[(size_t)i * n + c] = s / Lm[(size_t)i * n + i];
        }
    }
    return true;
}

}  // namespace

std::string mg_build(int K, int N, int Np, const int* etov, const double* geo, const int* conn,
                     const std::vector<double>& fc, const std::vector<int>& btype, double mass_coef,
                     const dgb::RefOps& ops, MgBuild& out) {
    out = MgBuild();
    int nv = 0;
    for (int q = 0; q < 3 * K; q++) nv = std::max(nv, etov[q] + 1);
    if (nv <= 0) return "no vertices";
    // barycentric coordinates of the nodes, ring order
    out.lam.resize((size_t)Np * 3);
    for (int p = 0; p < Np; p++) {
        const double r = ops.r[ops.ring[p]], s = ops.s[ops.ring[p]];
        out.lam[p * 3 + 0] = -(r + s) / 2;
        out.lam[p * 3 + 1] = (1 + r) / 2;
        out.lam[p * 3 + 2] = (1 + s) / 2;
    }
    // vertex -> element corners
    out.vptr.assign(nv + 1, 0);
    for (int q = 0; q < 3 * K; q++) out.vptr[etov[q] + 1]++;
    for (int v = 0; v < nv; v++) out.vptr[v + 1] += out.vptr[v];
    out.vinc.assign(3 * K, 0);
    {
        std::vector<int> fill(out.vptr.begin(), out.vptr.end() - 1);
        for (int q = 0; q < 3 * K; q++) out.vinc[fill[etov[q]]++] = q;
    }
    // level 0: P^T S P for continuous P1 functions
    std::vector<long long> key;
    std::vector<double> val;
    key.reserve((size_t)9 * K + 64);
    val.reserve((size_t)9 * K + 64);
    for (int k = 0; k < K; k++) {
        const double* g = geo + 4 * (size_t)k;
        const double rx = g[0], sx = g[1], ry = g[2], sy = g[3];
        const double J = 1.0 / (rx * sy - sx * ry);
        const double area = 2.0 * J;
        const double gx[3] = {-0.5 * (rx + sx), 0.5 * rx, 0.5 * sx};
        const double gy[3] = {-0.5 * (ry + sy), 0.5 * ry, 0.5 * sy};
        double a[3][3];
        for (int c = 0; c < 3; c++)
            for (int d = 0; d < 3; d++) {
                a[c][d] = area * (gx[c] * gx[d] + gy[c] * gy[d]);
                if (mass_coef != 0.0) a[c][d] += mass_coef * area / 12.0 * (c == d ? 2.0 : 1.0);
            }
        for (int f = 0; f < 3; f++) {
            const int cn = conn[(size_t)k * 3 + f];
            if (cn >= 0 || btype[-1 - cn] != 0) continue;
            // Nitsche terms of a fixed-value face: tau int u v - int (du/dn v + u dv/dn)
            const double* fk = &fc[((size_t)k * 3 + f) * kFaceCoef];
            const double tau = 2.0 * fk[4], len = 2.0 * fk[5];
            double nx, ny, fsc;
            face_normal(f, rx, sx, ry, sy, nx, ny, fsc);
            double dn[3], m1[3] = {0, 0, 0}, mf[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            for (int c = 0; c < 3; c++) dn[c] = nx * gx[c] + ny * gy[c];
            const int fa = f, fb = (f + 1) % 3;
            m1[fa] = m1[fb] = len / 2;
            mf[fa][fa] = mf[fb][fb] = len / 3;
            mf[fa][fb] = mf[fb][fa] = len / 6;
            for (int c = 0; c < 3; c++)
                for (int d = 0; d < 3; d++) a[c][d] += tau * mf[c][d] - (dn[c] * m1[d] + m1[c] * dn[d]);
        }
        for (int c = 0; c < 3; c++)
            for (int d = 0; d < 3; d++) {
                key.push_back((long long)etov[3 * k + c] * nv + etov[3 * k + d]);
                val.push_back(a[c][d]);
            }
    }
    out.levels.emplace_back();
    to_csr(nv, key, val, out.levels.back());
    jacobi_of(out.levels.back());
    // aggregation levels
    while (out.levels.back().n > kCoarsest) {
        if ((int)out.levels.size() >= kMgMaxLevels) return "too many levels";
        MgBuild::Level& F = out.levels.back();
        const int na = aggregate(F, F.agg);
        if (na > F.n * 9 / 10) return "aggregation does not coarsen";
        F.cptr.assign(na + 1, 0);
        for (int i = 0; i < F.n; i++) F.cptr[F.agg[i] + 1]++;
        for (int a = 0; a < na; a++) F.cptr[a + 1] += F.cptr[a];
        F.cmem.assign(F.n, 0);
        {
            std::vector<int> fill(F.cptr.begin(), F.cptr.end() - 1);
            for (int i = 0; i < F.n; i++) F.cmem[fill[F.agg[i]]++] = i;
        }
        key.clear();
        val.clear();
        for (int i = 0; i < F.n; i++)
            for (int q = F.rowptr[i]; q < F.rowptr[i + 1]; q++) {
                key.push_back((long long)F.agg[i] * na + F.agg[F.col[q]]);
                val.push_back(F.val[q]);
            }
        MgBuild::Level C;
        to_csr(na, key, val, C);
        jacobi_of(C);
        out.levels.push_back(std::move(C));
    }
    // coarsest: dense inverse
    const MgBuild::Level& C = out.levels.back();
    out.nc = C.n;
    out.Cinv.assign((size_t)C.n * C.n, 0.0);
    for (int i = 0; i < C.n; i++)
        for (int q = C.rowptr[i]; q < C.rowptr[i + 1]; q++) out.Cinv[(size_t)i * C.n + C.col[q]] = C.val[q];
    if (!spd_inverse(C.n, out.Cinv)) return "coarse operator is not positive definite";
    (void)N;
    return "";
}

// ---------------------------------------------------------------------------
// device cycle

__global__ void mg_restrict_dg_kernel(MgLevels m, const double* __restrict__ r, double* __restrict__ r1) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.lv[0].n) return;
    double s = 0;
    for (int q = m.vptr[v]; q < m.vptr[v + 1]; q++) {
        const int c = m.vinc[q], k = c / 3, lv = c - 3 * k;
        const double* rk = r + (size_t)k * m.Np;
        for (int i = 0; i < m.Np; i++) s += m.lam[i * 3 + lv] * rk[i];
    }
    r1[v] = s;
}

// x = dinv r
__global__ void mg_jacobi0_kernel(int n, const double* __restrict__ dinv, const double* __restrict__ r,
                                  double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = dinv[i] * r[i];
}

// t = r - A x
__global__ void mg_residual_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                   const double* __restrict__ val, const double* __restrict__ r,
                                   const double* __restrict__ x, double* __restrict__ t) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = r[i];
    for (int q = rowptr[i]; q < rowptr[i + 1]; q++) s -= val[q] * x[col[q]];
    t[i] = s;
}

// x += dinv (r - A x), the residual computed in the same pass into t
__global__ void mg_smooth_kernel(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
                                 const double* __restrict__ val, const double* __restrict__ dinv,
                                 const double* __restrict__ r, const double* __restrict__ x,
                                 double* __restrict__ xo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double s = r[i];
    for (int q = rowptr[i]; q < rowptr[i + 1]; q++) s -= val[q] * x[col[q]];
    xo[i] = x[i] + dinv[i] * s;
}

__global__ void mg_restrict_agg_kernel(int nc, const int* __restrict__ cptr, const int* __restrict__ cmem,
                                       const double* __restrict__ t, double* __restrict__ rc) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nc) return;
    double s = 0;
    for (int q = cptr[a]; q < cptr[a + 1]; q++) s += t[cmem[q]];
    rc[a] = s;
}

__global__ void mg_prolong_agg_kernel(int n, const int* __restrict__ agg, const double* __restrict__ xc,
                                      double* __restrict__ x) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] += xc[agg[i]];
}

// x = Cinv r, one warp per row
__global__ void mg_dense_kernel(int n, const double* __restrict__ Cinv, const double* __restrict__ r,
                                double* __restrict__ x) {
    const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0;
    for (int j = lane; j < n; j += 32) s += Cinv[(size_t)row * n + j] * r[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[row] = s;
}

// z = zb + P x1; r.z; dz mirror; finish like the learned preconditioner's collect
__global__ void mg_collect_kernel(MgLevels m, const double* __restrict__ zb, const double* __restrict__ x1,
                                  const double* __restrict__ r, double* __restrict__ z, float* __restrict__ dz,
                                  int mode, PcgScalars* S, double* part) {
    __shared__ double c0s[256];
    if (mode == 3 && S->done) return;
    const int Np = m.Np, EB = 256 / Np;
    const int e = threadIdx.x / Np, q = threadIdx.x - e * Np;
    const int ngroups = (m.K + EB - 1) / EB;
    double rz = 0;
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const int k = grp * EB + e;
        const bool act = e < EB && k < m.K;
        double c = 0;
        if (act) {
            const size_t t = (size_t)k * Np + q;
            c = m.lam[q * 3 + 0] * x1[m.etov[3 * (size_t)k]] + m.lam[q * 3 + 1] * x1[m.etov[3 * (size_t)k + 1]] +
                m.lam[q * 3 + 2] * x1[m.etov[3 * (size_t)k + 2]];
            const double zv = zb[t] + c;
            z[t] = zv;
            rz += r[t] * zv;
            if (q == 0) c0s[e] = c;
        }
        if (dz) {
            // dz enters as the offset mirror of zb: z - z0 = (zb - zb0) + (c - c0)
            __syncthreads();
            if (act) {
                const size_t t = (size_t)k * Np + q;
                dz[t] = dz[t] + (float)(c - c0s[e]);
            }
            __syncthreads();
        }
    }
    double val[1] = {rz}, tot[1];
    if (grid_sum<1>(val, part, gridDim.x, &S->counter, tot) && threadIdx.x == 0) {
        if (mode == 3) pcg_finish(S, tot[0], 0.0, S->rr);
        else S->rz = tot[0];
    }
}

static unsigned nb256(int n) { return (unsigned)((n + 255) / 256); }

cudaError_t launch_mg_correction(const MgLevels& m, const double* r, const double* zb, double* z, float* dz,
                                 int mode, PcgScalars* S, double* part, int grid, const int* done,
                                 cudaStream_t s) {
    (void)done;
    const int L = m.nl;
    mg_restrict_dg_kernel<<<nb256(m.lv[0].n), 256, 0, s>>>(m, r, m.lv[0].r);
    // down: pre-smooth, restrict the residual
    for (int l = 0; l + 1 < L; l++) {
        const MgLevel& a = m.lv[l];
        mg_jacobi0_kernel<<<nb256(a.n), 256, 0, s>>>(a.n, a.dinv, a.r, a.x);
        mg_residual_kernel<<<nb256(a.n), 256, 0, s>>>(a.n, a.rowptr, a.col, a.val, a.r, a.x, a.t);
        mg_restrict_agg_kernel<<<nb256(m.lv[l + 1].n), 256, 0, s>>>(m.lv[l + 1].n, a.cptr, a.cmem, a.t, m.lv[l + 1].r);
    }
    {
        const MgLevel& c = m.lv[L - 1];
        mg_dense_kernel<<<(c.n + 7) / 8, 256, 0, s>>>(c.n, m.Cinv, c.r, c.x);
    }
    // up: prolong the correction, post-smooth into t (the level's result: t
    // below the coarsest, x on the coarsest)
    for (int l = L - 2; l >= 0; l--) {
        const MgLevel& a = m.lv[l];
        const double* xc = (l + 1 == L - 1) ? m.lv[l + 1].x : m.lv[l + 1].t;
        mg_prolong_agg_kernel<<<nb256(a.n), 256, 0, s>>>(a.n, a.agg, xc, a.x);
        mg_smooth_kernel<<<nb256(a.n), 256, 0, s>>>(a.n, a.rowptr, a.col, a.val, a.dinv, a.r, a.x, a.t);
    }
    const double* x1 = (L == 1) ? m.lv[0].x : m.lv[0].t;
    const int EB = 256 / m.Np;
    const int ngroups = (m.K + EB - 1) / EB;
    mg_collect_kernel<<<std::min(ngroups, grid), 256, 0, s>>>(m, zb, x1, r, z, dz, mode, S, part);
    return cudaGetLastError();
}

}  // namespace dgk
