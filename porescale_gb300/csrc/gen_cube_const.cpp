// gen_cube_const.cpp -- writes lsm_cube_const.h: the cube stiffness matrices
// per unit alpha and per unit beta (lsm_cube.h) as compile-time constants,
// so that the FP32 matvec multiplies by literal values and the compiler
// drops the zero entries (Ka has 192 and Kb 456 nonzeros of 576).  Every
// entry is a multiple of 1/8 up to rounding of the construction; the
// generator prints the exact doubles.  It also prints the stencil of a node
// whose 8 cubes are all solid and of one material: the sum over those cubes
// of the blocks coupling the node to each of its 27 box neighbours.  Those
// sums are multiples of 1/8 (0 where the terms cancel) up to the
// construction's rounding, and are printed as the exact multiples, so that
// the bulk stencil is exactly symmetric under d -> -d and its rows sum to
// exactly zero.  Regenerate with
//   g++ -O2 -I. gen_cube_const.cpp -o gen && ./gen > lsm_cube_const.h
// (tests/test_oracle_cpu.py checks that the committed header is current).
#include <cmath>
#include <cstdio>

#include "lsm_cube.h"

int main()
{
  ps::lsm::CubeMatrices M;
  ps::lsm::build_cube_matrices(M);
  std::printf("// lsm_cube_const.h -- generated by gen_cube_const.cpp from lsm_cube.h; do not edit.\n");
  std::printf("// Cube stiffness per unit alpha (Ka) and per unit beta (Kb), corner c of the\n");
  std::printf("// cube at offset (c&1, (c>>1)&1, c>>2), rows / columns 3 c + component.\n");
  std::printf("#pragma once\n\nnamespace ps {\nnamespace lsm {\n\n");
  const char* names[2] = {"kCubeKa", "kCubeKb"};
  for (int k = 0; k < 2; k++) {
    std::printf("constexpr double %s[24][24] = {\n", names[k]);
    for (int i = 0; i < 24; i++) {
      std::printf("    {");
      for (int j = 0; j < 24; j++) std::printf("%.17g%s", k == 0 ? M.Ka[i][j] : M.Kb[i][j], j < 23 ? ", " : "");
      std::printf("}%s\n", i < 23 ? "," : "");
    }
    std::printf("};\n\n");
  }
  std::printf("// Bulk stencil per unit alpha (kBulkKa) and per unit beta (kBulkKb): entry\n");
  std::printf("// [d][3 r + c] couples component r of a node to component c of its\n");
  std::printf("// neighbour at offset (dx, dy, dz) = (d %% 3, d / 3 %% 3, d / 9) - 1, summed\n");
  std::printf("// over the node's 8 cubes.\n");
  for (int k = 0; k < 2; k++) {
    double S[27][9] = {};
    for (int e = 0; e < 8; e++)  // the cube whose corner e is the node
      for (int b = 0; b < 8; b++) {
        const int dx = (b & 1) - (e & 1), dy = ((b >> 1) & 1) - ((e >> 1) & 1), dz = (b >> 2) - (e >> 2);
        const int d = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1);
        for (int r = 0; r < 3; r++)
          for (int c = 0; c < 3; c++) S[d][3 * r + c] += k == 0 ? M.Ka[3 * e + r][3 * b + c] : M.Kb[3 * e + r][3 * b + c];
      }
    std::printf("constexpr double %s[27][9] = {\n", k == 0 ? "kBulkKa" : "kBulkKb");
    for (int d = 0; d < 27; d++) {
      std::printf("    {");
      for (int j = 0; j < 9; j++) {
        const double e = std::nearbyint(8.0 * S[d][j]) / 8.0;
        if (std::fabs(e - S[d][j]) > 1e-9) return 1;  // not a multiple of 1/8
        std::printf("%.17g%s", e == 0.0 ? 0.0 : e, j < 8 ? ", " : "");
      }
      std::printf("}%s\n", d < 26 ? "," : "");
    }
    std::printf("};\n\n");
  }
  std::printf("}  // namespace lsm\n}  // namespace ps\n");
  return 0;
}
