// Host finite-element math of the hexahedral element, shared by the library
// (setup.cu, fine.cu) and the build-time generator of the default-material
// stencil table (gen_default_stencil.cu): both compute the same numbers
// through the same code.
#pragma once

#include <algorithm>
#include <cmath>
#include <vector>

#include "gmgs_internal.cuh"

namespace gmgs {

// ---------------------------------------------------------------------------
// host FEM math (SetupStiffnessMatrix.m, ElementElasticityMatrix.m,
// ElementStrainMatrix.m, GaussianIntegral.m, ShapeFunction.m,
// DeShapeFunction.m, GetCartesianStress.m:44-73)
// ---------------------------------------------------------------------------
inline constexpr double kGauss = 0.577350269189626;   // GaussianIntegral.m:11 writes 15 digits
inline constexpr int kSign[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                                {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};

inline void hooke(double E, double nu, double S[6][6]) {
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) S[i][j] = 0;
    const double c1 = (1 + nu) * (1 - 2 * nu), c2 = 2 * (1 + nu);
    S[0][0] = E * (1 - nu) / c1;
    S[0][1] = E * nu / c1;
    S[0][2] = S[0][1];
    S[1][0] = S[0][1]; S[1][1] = S[0][0]; S[1][2] = S[1][0];
    S[2][0] = S[0][2]; S[2][1] = S[1][2]; S[2][2] = S[1][1];
    S[3][3] = E / c2; S[4][4] = S[3][3]; S[5][5] = S[4][4];
}

inline bool invert(int n, const double* A, double* Ainv) {
    std::vector<double> M(A, A + n * n), I(n * n, 0.0);
    for (int i = 0; i < n; ++i) I[i * n + i] = 1;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(M[r * n + c]) > std::fabs(M[piv * n + c])) piv = r;
        if (M[piv * n + c] == 0) return false;
        if (piv != c)
            for (int k = 0; k < n; ++k) { std::swap(M[c * n + k], M[piv * n + k]); std::swap(I[c * n + k], I[piv * n + k]); }
        const double d = M[c * n + c];
        for (int k = 0; k < n; ++k) { M[c * n + k] /= d; I[c * n + k] /= d; }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const double f = M[r * n + c];
            if (f == 0) continue;
            for (int k = 0; k < n; ++k) { M[r * n + k] -= f * M[c * n + k]; I[r * n + k] -= f * I[c * n + k]; }
        }
    }
    std::copy(I.begin(), I.end(), Ainv);
    return true;
}

// B (48x24) and the Jacobian determinants of a box element with edge lengths
// (dx, dy, dz); node 1 at (-x, -y, -z) (DiscretizeDesignDomain.m:96).
inline void strain_matrix(const double ele[3], double B[48][24], double detJ[8]) {
    double X[8][3];
    for (int k = 0; k < 8; ++k)
        for (int d = 0; d < 3; ++d) X[k][d] = (kSign[k][d] + 1) * 0.5 * ele[d];
    for (int g = 0; g < 48; ++g)
        for (int j = 0; j < 24; ++j) B[g][j] = 0;
    for (int g = 0; g < 8; ++g) {
        const double s = kGauss * kSign[g][0], t = kGauss * kSign[g][1], p = kGauss * kSign[g][2];
        double dN[3][8];
        for (int k = 0; k < 8; ++k) {
            const double fs = 1 + s * kSign[k][0], ft = 1 + t * kSign[k][1], fp = 1 + p * kSign[k][2];
            dN[0][k] = 0.125 * kSign[k][0] * ft * fp;
            dN[1][k] = 0.125 * kSign[k][1] * fs * fp;
            dN[2][k] = 0.125 * kSign[k][2] * fs * ft;
        }
        double J[9], Ji[9];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                double v = 0;
                for (int k = 0; k < 8; ++k) v += dN[a][k] * X[k][b];
                J[a * 3 + b] = v;
            }
        detJ[g] = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                  J[2] * (J[3] * J[7] - J[4] * J[6]);
        invert(3, J, Ji);
        for (int k = 0; k < 8; ++k) {
            double d[3];
            for (int a = 0; a < 3; ++a) d[a] = Ji[a * 3 + 0] * dN[0][k] + Ji[a * 3 + 1] * dN[1][k] + Ji[a * 3 + 2] * dN[2][k];
            const int r = 6 * g, c = 3 * k;
            B[r + 0][c + 0] = d[0];
            B[r + 1][c + 1] = d[1];
            B[r + 2][c + 2] = d[2];
            B[r + 3][c + 1] = d[2]; B[r + 3][c + 2] = d[1];
            B[r + 4][c + 0] = d[2]; B[r + 4][c + 2] = d[0];
            B[r + 5][c + 0] = d[1]; B[r + 5][c + 1] = d[0];
        }
    }
}

inline void element_stiffness(double E, double nu, const double ele[3], double Ke[576]) {
    double B[48][24];
    double detJ[8], S[6][6];
    strain_matrix(ele, B, detJ);
    hooke(E, nu, S);
    // (B^T (D .* wgt)) B, the reference's evaluation order (SetupStiffnessMatrix.m:22)
    std::vector<double> BtDw(24 * 48, 0.0);
    for (int i = 0; i < 24; ++i)
        for (int g = 0; g < 8; ++g)
            for (int b = 0; b < 6; ++b) {
                double v = 0;
                for (int a = 0; a < 6; ++a) v += B[6 * g + a][i] * S[a][b];
                BtDw[i * 48 + 6 * g + b] = v * detJ[g];
            }
    for (int i = 0; i < 24; ++i)
        for (int j = 0; j < 24; ++j) {
            double v = 0;
            for (int r = 0; r < 48; ++r) v += BtDw[i * 48 + r] * B[r][j];
            Ke[i * 24 + j] = v;
        }
}


// The assembled interior stencil of a uniform grid from the element matrix
// (row = output DOF): S[k][3a + b] = sum over the 8 elements around a node of
// the coupling between the node and its neighbour at offset k
// (k = (dz+1)*9 + (dx+1)*3 + (dy+1)).
inline void stencil_from_rows(const double* ke_rows, double S[27][9]) {
    for (int k = 0; k < 27; ++k)
        for (int i = 0; i < 9; ++i) S[k][i] = 0.0;
    for (int k = 0; k < 27; ++k) {
        const int dy = k % 3 - 1, dx = (k / 3) % 3 - 1, dz = k / 9 - 1;
        for (int e = 0; e < 8; ++e) {
            const int A = e & 1, B = (e >> 1) & 1, C = e >> 2;     // node = element origin + (A, B, C)
            const int my = A + dy, mx = B + dx, mz = C + dz;       // neighbour relative to the origin
            if (my < 0 || my > 1 || mx < 0 || mx > 1 || mz < 0 || mz > 1) continue;
            const int cn = corner_of(A, B, C), cm = corner_of(my, mx, mz);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) S[k][3 * a + b] += ke_rows[(3 * cn + a) * 24 + 3 * cm + b];
        }
    }
}

}  // namespace gmgs
