// mg.hpp -- multilevel (coarse-space) correction for the SIPG block-Jacobi PCG.
//
// Preconditioner  z = B r + P V(P^T r):  B the block-Jacobi inverse, P the
// prolongation of continuous piecewise-linear functions on the mesh vertices
// into the DG space (exact: P1 is inside P_N), V one symmetric V(1,1) cycle
// on the Galerkin coarse operator A_1 = P^T S P (assembled in closed form: for
// continuous P1 functions the interior-face terms of SIPG vanish, leaving the
// P1 stiffness, the Nitsche terms of the fixed-value boundary faces and the
// Helmholtz mass term), weighted-Jacobi smoothing, coarser levels by greedy
// vertex aggregation with piecewise-constant transfer, the coarsest solved by
// a dense inverse.  Everything is linear and symmetric, so plain PCG applies.
#pragma once

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "dg_basis.hpp"
#include "ipdg.hpp"

namespace dgk {

constexpr int kMgMaxLevels = 10;

struct MgLevel {
    int n = 0;
    const int* rowptr = nullptr;  // A_l in CSR
    const int* col = nullptr;
    const double* val = nullptr;
    const double* dinv = nullptr;  // omega / diag(A_l)
    // transfer to level l + 1 (null on the coarsest level)
    const int* agg = nullptr;      // [n] coarse index of each unknown
    const int* cptr = nullptr;     // coarse -> members (CSR), deterministic restriction
    const int* cmem = nullptr;
    double* r = nullptr;           // work vectors of the cycle
    double* x = nullptr;
    double* t = nullptr;
};

struct MgLevels {
    int nl = 0;                    // levels lv[0] (P1 on the vertices) .. lv[nl-1] (the coarsest)
    MgLevel lv[kMgMaxLevels];
    const double* Cinv = nullptr;  // dense inverse of the coarsest operator (row-major)
    int K = 0, Np = 0;
    const int* etov = nullptr;     // [K][3] vertex ids
    const double* lam = nullptr;   // [Np][3] barycentric coordinates of the nodes (ring order)
    const int* vptr = nullptr;     // vertex -> incident element corners k*3+c (CSR)
    const int* vinc = nullptr;
};

// host-side levels
struct MgBuild {
    struct Level {
        int n = 0;
        std::vector<int> rowptr, col, agg, cptr, cmem;
        std::vector<double> val, dinv;
    };
    std::vector<int> vptr, vinc;
    std::vector<double> lam;
    std::vector<Level> levels;  // levels[0]: P1 on the vertices
    std::vector<double> Cinv;
    int nc = 0;
};

// Builds the levels; "" on success.  etov: [K][3] vertex ids, geo: [K][4]
// metrics, conn: packed neighbours (negative: boundary slot), fc: the face
// coefficients as built (tau/2 and sJ per element face), btype: per
// boundary slot (0: fixed value, Nitsche terms; otherwise none), mass_coef:
// Helmholtz coefficient.
std::string mg_build(int K, int N, int Np, const int* etov, const double* geo, const int* conn,
                     const std::vector<double>& fc, const std::vector<int>& btype, double mass_coef,
                     const dgb::RefOps& ops, MgBuild& out);

// z = zb + P V(P^T r) with r.z reduced like the learned preconditioner's
// collect step (mode: 1 init -> S->rz, 2 refresh -> S->rz, 3 iteration ->
// pcg_finish); dz (mixed precision) is completed as an offset mirror
cudaError_t launch_mg_correction(const MgLevels& m, const double* r, const double* zb, double* z, float* dz,
                                 int mode, PcgScalars* S, double* part, int grid, const int* done,
                                 cudaStream_t s);

}  // namespace dgk
