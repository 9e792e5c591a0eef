// Build-time generator (host only): the FP32 stencil and element-matrix
// tables of the streaming kernels for the reference's default material and
// voxel (E = 1, nu = 0.3, 1 x 1 x 1; GlobalVariables.m:3-23), written as
// constexpr functions so the kernels compiled for them carry the
// coefficients as instruction immediates instead of loading them per plane.
// The values come from the library's own element_stiffness and
// stencil_from_rows (element_host.h) and the same float rounding as
// make_stencil; at run time a model's coefficients are compared with these
// bit for bit before the specialised kernels are used.
//
//     gen_default_stencil <output header>
#include <cstdio>

#include "element_host.h"

int main(int argc, char** argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: gen_default_stencil <header>\n");
        return 2;
    }
    const double ele[3] = {1.0, 1.0, 1.0};
    double Ke[gmgs::KE], KeT[gmgs::KE];
    gmgs::element_stiffness(1.0, 0.3, ele, Ke);
    for (int i = 0; i < 24; ++i)
        for (int j = 0; j < 24; ++j) KeT[i * 24 + j] = Ke[j * 24 + i];   // row = output DOF
    double S[27][9];
    gmgs::stencil_from_rows(KeT, S);
    std::FILE* f = std::fopen(argv[1], "w");
    if (!f) return 1;
    std::fprintf(f, "// generated by gen_default_stencil.cu: FP32 stencil (S) and element matrix (K) of\n"
                    "// E = 1, nu = 0.3, 1 x 1 x 1 voxels\n#pragma once\nnamespace gmgs {\nnamespace dflt {\n");
    std::fprintf(f, "__host__ __device__ constexpr float S(int i) {\n    switch (i) {\n");
    for (int k = 0; k < 27; ++k)
        for (int i = 0; i < 9; ++i) std::fprintf(f, "    case %d: return %af;\n", k * 9 + i, (double)(float)S[k][i]);
    std::fprintf(f, "    default: return 0.0f;\n    }\n}\n");
    std::fprintf(f, "__host__ __device__ constexpr float K(int i) {\n    switch (i) {\n");
    for (int i = 0; i < gmgs::KE; ++i) std::fprintf(f, "    case %d: return %af;\n", i, (double)(float)KeT[i]);
    std::fprintf(f, "    default: return 0.0f;\n    }\n}\n}  // namespace dflt\n}  // namespace gmgs\n");
    return std::fclose(f) == 0 ? 0 : 1;
}
