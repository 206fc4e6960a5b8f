// dg_basis.hpp -- host-side (FP64) reference-element operators for the GPU path.
//
// Builds, once per order, the nodal basis of HopeFOAM's triangle element and
// the fused matrices the kernels apply:
//   nodes: warp & blend with the alpha table of
//     element/baseFunctions/straightBaseFunctions/triangleBaseFunction/triangleBaseFunction.C:122-186
//   V, Dr, Ds: orthonormal Dubiner basis (element/polynomials/Legendre/Legendre.C:273-310, :387-450)
//   cubature interpolation / derivatives at the strength-3(N+1) rule and the
//     (N+2)-point face Gauss rule (element/gaussIntegration/gaussTriangleIntegration/
//     gaussTriangleIntegration.C:45-97)
// and the fused forms used on straight-sided (affine) triangles, where the
// per-element mass matrix is J * Mref:
//   Sr = Mref^-1 Dr_g^T W, Ss = Mref^-1 Ds_g^T W        (volume term, no J)
//   Lift[:, f*Nfq + i] = Mref^-1 I_f^T w_i on face f     (scaled by sJ/J per face)
// Node storage order on the device is the "ring" order: the 3N boundary nodes
// first, walking faces 0, 1, 2 in their own direction, then the interior
// nodes; face f's Nfp nodes are ring positions (f*N + j) mod 3N.
#pragma once

#include <string>
#include <vector>

namespace dgb {

int cubature_points_for_order(int N);  // expected rule size (0 if unknown)

struct RefOps {
    int N = 0, Np = 0, Nfp = 0, Ng = 0, Nfq = 0;
    std::vector<double> r, s;          // nodes, reference order
    std::vector<int> ring;             // ring position -> reference node id
    std::vector<int> fnode;            // [3][Nfp] reference node id of face node j (face direction)
    std::vector<double> V, invV, Dr, Ds;    // Np x Np, reference order
    std::vector<double> gr, gs, gw;    // cubature
    std::vector<double> Vg, Drg, Dsg;  // Ng x Np, reference order
    std::vector<double> fq, fw;        // face Gauss rule
    std::vector<double> If;            // Nfq x Nfp face interpolation (face direction)
    std::vector<double> Mref, Minv;    // Np x Np reference mass matrix (J = 1) and inverse
    // fused device operators, ring order
    std::vector<double> dVg;           // Ng x Np
    std::vector<double> dSr, dSs;      // Np x Ng
    std::vector<double> dLift;         // Np x 3Nfq
};

// Returns "" on success, else an error message.
std::string build_ref_ops(int N, const double* cub, int Ng, RefOps& ops);

}  // namespace dgb
