// gen_cube_const.cpp -- writes lsm_cube_const.h: the cube stiffness matrices
// per unit alpha and per unit beta (lsm_cube.h) as compile-time constants,
// so that the FP32 matvec multiplies by literal values and the compiler
// drops the zero entries (Ka has 192 and Kb 456 nonzeros of 576).  Every
// entry is a multiple of 1/8 up to rounding of the construction; the
// generator prints the exact doubles.  Regenerate with
//   g++ -O2 -I. gen_cube_const.cpp -o gen && ./gen > lsm_cube_const.h
// (tests/test_oracle_cpu.py checks that the committed header is current).
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
  std::printf("}  // namespace lsm\n}  // namespace ps\n");
  return 0;
}
