// Continuous P1 / P2 Lagrange basis on triangles (ExtendableFEMBase H1P1,
// H1P2 on Triangle2D): local dofs are the three vertices, then (P2) the
// midpoints of the faces (1,2), (2,3), (3,1).  Values and gradients are
// written in terms of the barycentric coordinates lam and their constant
// gradients g = (grad lam_0, grad lam_1, grad lam_2) (6 doubles).
#pragma once

namespace sgfem_fe {

__host__ __device__ __forceinline__ int ndofs4cell(int order) { return order == 1 ? 3 : 6; }

__host__ __device__ __forceinline__ void basis_val(int order, const double* lam, double* out) {
    if (order == 1) {
        out[0] = lam[0];
        out[1] = lam[1];
        out[2] = lam[2];
        return;
    }
    const int ea[3] = {0, 1, 2}, eb[3] = {1, 2, 0};
    for (int i = 0; i < 3; ++i) out[i] = lam[i] * (2.0 * lam[i] - 1.0);
    for (int e = 0; e < 3; ++e) out[3 + e] = 4.0 * lam[ea[e]] * lam[eb[e]];
}

// gradients (2 per local dof) at barycentric lam
__host__ __device__ __forceinline__ void basis_grad(int order, const double* g, const double* lam, double* out) {
    if (order == 1) {
        for (int i = 0; i < 6; ++i) out[i] = g[i];
        return;
    }
    const int ea[3] = {0, 1, 2}, eb[3] = {1, 2, 0};
    for (int i = 0; i < 3; ++i) {
        out[2 * i] = (4.0 * lam[i] - 1.0) * g[2 * i];
        out[2 * i + 1] = (4.0 * lam[i] - 1.0) * g[2 * i + 1];
    }
    for (int e = 0; e < 3; ++e) {
        const int a = ea[e], b = eb[e];
        out[6 + 2 * e] = 4.0 * (lam[a] * g[2 * b] + lam[b] * g[2 * a]);
        out[6 + 2 * e + 1] = 4.0 * (lam[a] * g[2 * b + 1] + lam[b] * g[2 * a + 1]);
    }
}

}  // namespace sgfem_fe
