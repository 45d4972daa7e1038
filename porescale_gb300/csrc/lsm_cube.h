// lsm_cube.h -- the lattice-spring model of one voxel cube, as matrices.
//
// The reference assembles its spring network from per-node bond and angle
// tables whose constants count the adjacent solid cubes (XX_P.f:626-1261):
// an edge bond gets 1/4 of alpha per adjacent solid cube, a face diagonal
// 1/2, a pi/4 angle 1/2 of beta per cube sharing its plane, a pi/3 angle the
// full beta of its one cube.  The same network is the sum over solid cubes
// of one cube's 24 bonds (12 edges at 1/4, 12 face diagonals at 1/2) and 72
// angles (48 pi/4 at 1/2, 24 pi/3 at 1) with that cube's alpha and beta --
// the decomposition the reference's calc_stress uses (XX_P.f:1761-1957).
//
// Both spring kinds are linear in the displacements:
//   bond a-b, unit direction n:  force on a = w alpha ((u_b - u_a).n) n
//   angle (i; j, k):  theta = (u_j - u_i).f_j + (u_k - u_i).f_k with
//     f_j = n x c_j / |c_j|^2, f_k = -(n x c_k) / |c_k|^2, n the unit normal
//     of the angle's plane; force = -w beta theta grad(theta)
// so a cube contributes K = alpha K_a + beta K_b (24 x 24, symmetric, PSD)
// to the stiffness, and the reference's cube stress sigma+ (calc_stress) is
// S = alpha S_a + beta S_b applied to the 8 corner displacements (9 x 24).
// Corner c of a cube sits at offset (c&1, (c>>1)&1, (c>>2)&1).
#pragma once
#include <cmath>
#include <cstring>

namespace ps {
namespace lsm {

// D3Q19 directions (reference `velocities19` order, 0-based) and the 9
// bond vectors (`velocities9` order)
static const int kCV[19][3] = {{0, 0, 0},  {1, 0, 0},  {-1, 0, 0}, {0, 1, 0},  {0, -1, 0}, {0, 0, 1},  {0, 0, -1},
                               {1, 1, 0},  {-1, 1, 0}, {1, -1, 0}, {-1, -1, 0}, {1, 0, 1},  {-1, 0, 1}, {1, 0, -1},
                               {-1, 0, -1}, {0, 1, 1},  {0, -1, 1}, {0, 1, -1}, {0, -1, -1}};
static const int kIB[9][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, -1, 0},
                              {1, 0, 1}, {1, 0, -1}, {0, 1, 1}, {0, 1, -1}};
// arm directions (1-based D3Q19 indices) of the 48 node angles: eight pi/4
// angles walking around each coordinate plane, then four pi/3 angles around
// each of the six face-diagonal cones (the reference's nta table)
static const int kNTA[48][2] = {
    {2, 8},   {8, 4},   {4, 9},   {9, 3},   {3, 11},  {11, 5},  {5, 10},  {10, 2},  {2, 12},  {12, 6},
    {6, 13},  {13, 3},  {3, 15},  {15, 7},  {7, 14},  {14, 2},  {4, 16},  {16, 6},  {6, 17},  {17, 5},
    {5, 19},  {19, 7},  {7, 18},  {18, 4},  {12, 16}, {16, 13}, {13, 17}, {17, 12}, {14, 18}, {18, 15},
    {15, 19}, {19, 14}, {8, 12},  {12, 10}, {10, 14}, {14, 8},  {9, 13},  {13, 11}, {11, 15}, {15, 9},
    {8, 16},  {16, 9},  {9, 18},  {18, 8},  {10, 17}, {17, 11}, {11, 19}, {19, 10}};

struct CubeMatrices {
  double Ka[24][24], Kb[24][24];  // stiffness per unit alpha / beta
  double Sa[9][24], Sb[9][24];    // sigma+ (row d*3+col) per unit alpha / beta
  int nbond, nangle;
};

inline void cross(const double* a, const double* b, double* c)
{
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

inline int corner_of(int x, int y, int z) { return x + 2 * y + 4 * z; }

inline void build_cube_matrices(CubeMatrices& M)
{
  std::memset(&M, 0, sizeof M);
  // bonds
  for (int a = 0; a < 8; a++)
    for (int j = 0; j < 9; j++) {
      const int bx = (a & 1) + kIB[j][0], by = ((a >> 1) & 1) + kIB[j][1], bz = ((a >> 2) & 1) + kIB[j][2];
      if (bx < 0 || bx > 1 || by < 0 || by > 1 || bz < 0 || bz > 1) continue;
      const int b = corner_of(bx, by, bz);
      const double w = j < 3 ? 0.25 : 0.5;
      double n[3];
      const double len = std::sqrt((double)(kIB[j][0] * kIB[j][0] + kIB[j][1] * kIB[j][1] + kIB[j][2] * kIB[j][2]));
      for (int d = 0; d < 3; d++) n[d] = kIB[j][d] / len;
      for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++) {
          const double k = w * n[p] * n[q];
          M.Ka[3 * a + p][3 * a + q] += k;
          M.Ka[3 * b + p][3 * b + q] += k;
          M.Ka[3 * a + p][3 * b + q] -= k;
          M.Ka[3 * b + p][3 * a + q] -= k;
        }
      // sigma+: the bond force on its first end, f = w ((u_b-u_a).n) n,
      // enters column `col` with the sign of n[col]
      for (int col = 0; col < 3; col++) {
        if (n[col] == 0.0) continue;
        const double sg = n[col] > 0 ? 1.0 : -1.0;
        for (int d = 0; d < 3; d++)
          for (int q = 0; q < 3; q++) {
            const double c = sg * w * n[d] * n[q];
            M.Sa[3 * d + col][3 * b + q] += c;
            M.Sa[3 * d + col][3 * a + q] -= c;
          }
      }
      M.nbond++;
    }
  // angles
  for (int a = 0; a < 8; a++)
    for (int j = 0; j < 48; j++) {
      const int* cj = kCV[kNTA[j][0] - 1];
      const int* ck = kCV[kNTA[j][1] - 1];
      const int p[3] = {a & 1, (a >> 1) & 1, (a >> 2) & 1};
      const int qj[3] = {p[0] + cj[0], p[1] + cj[1], p[2] + cj[2]};
      const int qk[3] = {p[0] + ck[0], p[1] + ck[1], p[2] + ck[2]};
      bool in = true;
      for (int d = 0; d < 3; d++) in = in && qj[d] >= 0 && qj[d] <= 1 && qk[d] >= 0 && qk[d] <= 1;
      if (!in) continue;
      const int bj = corner_of(qj[0], qj[1], qj[2]), bk = corner_of(qk[0], qk[1], qk[2]);
      const double w = j >= 24 ? 1.0 : 0.5;
      double vj[3], vk[3], n[3], fj[3], fk[3];
      for (int d = 0; d < 3; d++) {
        vj[d] = cj[d];
        vk[d] = ck[d];
      }
      cross(vj, vk, n);
      const double nn = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int d = 0; d < 3; d++) n[d] /= nn;
      const double j2 = vj[0] * vj[0] + vj[1] * vj[1] + vj[2] * vj[2], k2 = vk[0] * vk[0] + vk[1] * vk[1] + vk[2] * vk[2];
      cross(n, vj, fj);
      cross(n, vk, fk);
      for (int d = 0; d < 3; d++) {
        fj[d] /= j2;
        fk[d] = -fk[d] / k2;
      }
      // grad theta over the three corners
      double g[3][3];
      int node[3] = {a, bj, bk};
      for (int d = 0; d < 3; d++) {
        g[0][d] = -(fj[d] + fk[d]);
        g[1][d] = fj[d];
        g[2][d] = fk[d];
      }
      for (int s = 0; s < 3; s++)
        for (int t = 0; t < 3; t++)
          for (int p2 = 0; p2 < 3; p2++)
            for (int q2 = 0; q2 < 3; q2++) M.Kb[3 * node[s] + p2][3 * node[t] + q2] += w * g[s][p2] * g[t][q2];
      // sigma+: the reference adds -dfi*f_j to column col by the sign of arm
      // j's direction (and likewise for k), with dfi = -w beta theta
      const int dirs[2][3] = {{cj[0], cj[1], cj[2]}, {ck[0], ck[1], ck[2]}};
      const double* fv[2] = {fj, fk};
      for (int arm = 0; arm < 2; arm++)
        for (int col = 0; col < 3; col++) {
          if (dirs[arm][col] == 0) continue;
          const double sg = dirs[arm][col] > 0 ? 1.0 : -1.0;
          for (int d = 0; d < 3; d++)
            for (int s = 0; s < 3; s++)
              for (int q2 = 0; q2 < 3; q2++) M.Sb[3 * d + col][3 * node[s] + q2] += sg * w * fv[arm][d] * g[s][q2];
        }
      M.nangle++;
    }
}

}  // namespace lsm
}  // namespace ps
