// Compile-time lattice stencil families for the tiled FP32 kernels.
//
// A family fixes, for every basis site b, the list of neighbour slots
// (dX, dY, dZ, bj) in tile coordinates and how the slots group into
// isotropic shells.  The exchange constants (one J per shell, plus an
// optional 3x3 remainder per slot) stay runtime data.  The host matches an
// exchange interaction template against each family; anything else runs on
// the generic gather kernels.
//
// Tile coordinates: X is the streamed (slowest) axis, Z the fastest.  3-D
// families map (X, Y, Z) = (a1, a2, a3); 2-D (monolayer, L3 = 1) families map
// (X, Y, Z) = (a1, a3, a2) so that Z is the contiguous axis.
#pragma once

#include <cstdint>

namespace jams_llg {

struct Slot {
  int dx, dy, dz, bj;
};

enum FamilyId { kFamNone = 0, kFamSC = 1, kFamBCC = 2, kFamBCC3 = 3, kFamTRI = 4, kFamFCC = 5, kFamFCC2 = 6 };

// simple cubic, 6 nearest neighbours, one shell
// SEP: 0 plain slot gather; 1 bcc shell 1 as two carried 2x2 plane sums;
// 2 also shells 2 and 3 from carried in-plane cross sums (llg_tiled.cuh).
// bcc three shells use 2 (12 % faster at 256^3); bcc nearest neighbours
// keep the plain gather.
struct FamSC {
  static constexpr int id = kFamSC, SEP = 0;
  static constexpr int NB = 1, RX = 1, RY = 1, RZ = 1, TWO_D = 0;
  static constexpr int NSHELL = 1, Z = 6, REST = 0;
  __host__ __device__ static constexpr int shell_end(int /*b*/, int g) { return g == 0 ? 6 : 6; }
  __host__ __device__ static constexpr Slot slot(int /*b*/, int k) {
    return k == 0 ? Slot{1, 0, 0, 0} : k == 1 ? Slot{-1, 0, 0, 0} : k == 2 ? Slot{0, 1, 0, 0}
         : k == 3 ? Slot{0, -1, 0, 0} : k == 4 ? Slot{0, 0, 1, 0} : Slot{0, 0, -1, 0};
  }
};

// bcc as a 2-site conventional cubic cell: shell 1 = the 8 body-diagonal
// neighbours on the other sublattice
__host__ __device__ constexpr Slot bcc_shell1(int b, int k) {
  // b = 0: cells {-1, 0}^3 of sublattice 1; b = 1: cells {0, 1}^3 of sublattice 0
  return b == 0 ? Slot{-(k >> 2 & 1), -(k >> 1 & 1), -(k & 1), 1} : Slot{(k >> 2 & 1), (k >> 1 & 1), (k & 1), 0};
}

__host__ __device__ constexpr Slot bcc_shell2(int b, int k) {
  return k == 0 ? Slot{1, 0, 0, b} : k == 1 ? Slot{-1, 0, 0, b} : k == 2 ? Slot{0, 1, 0, b}
       : k == 3 ? Slot{0, -1, 0, b} : k == 4 ? Slot{0, 0, 1, b} : Slot{0, 0, -1, b};
}

__host__ __device__ constexpr Slot bcc_shell3(int b, int k) {
  // 12 face diagonals (+-1, +-1) in each of the planes xy, xz, yz
  return k < 4 ? Slot{(k & 1) ? -1 : 1, (k & 2) ? -1 : 1, 0, b}
       : k < 8 ? Slot{(k & 1) ? -1 : 1, 0, (k & 2) ? -1 : 1, b}
               : Slot{0, (k & 1) ? -1 : 1, (k & 2) ? -1 : 1, b};
}

struct FamBCC {
  static constexpr int id = kFamBCC, SEP = 0;   // SEP = 1 measured 2 % slower: too little to save
  static constexpr int NB = 2, RX = 1, RY = 1, RZ = 1, TWO_D = 0;
  static constexpr int NSHELL = 1, Z = 8, REST = 0;
  __host__ __device__ static constexpr int shell_end(int /*b*/, int /*g*/) { return 8; }
  __host__ __device__ static constexpr Slot slot(int b, int k) { return bcc_shell1(b, k); }
};

struct FamBCC3 {
  static constexpr int id = kFamBCC3, SEP = 2;
  static constexpr int NB = 2, RX = 1, RY = 1, RZ = 1, TWO_D = 0;
  static constexpr int NSHELL = 3, Z = 26, REST = 0;
  __host__ __device__ static constexpr int shell_end(int /*b*/, int g) { return g == 0 ? 8 : g == 1 ? 14 : 26; }
  __host__ __device__ static constexpr Slot slot(int b, int k) {
    return k < 8 ? bcc_shell1(b, k) : k < 14 ? bcc_shell2(b, k - 8) : bcc_shell3(b, k - 14);
  }
};

// fcc as a 4-site conventional cubic cell, sites at (0,0,0), (0,1/2,1/2),
// (1/2,0,1/2), (1/2,1/2,0).  fcc_half: twice the fractional coordinate of
// site b along axis.
__host__ __device__ constexpr int fcc_half(int b, int axis) { return b == 0 ? 0 : (b - 1 == axis ? 0 : 1); }

// shell 1: the 12 neighbours at a / sqrt(2), on the other three
// sublattices, in (partner, dX, dY, dZ) lexicographic order
__host__ __device__ constexpr Slot fcc_shell1(int b, int k) {
  int n = 0;
  for (int bj = 0; bj < 4; ++bj)
    for (int tx = -1; tx <= 1; ++tx)
      for (int ty = -1; ty <= 1; ++ty)
        for (int tz = -1; tz <= 1; ++tz) {
          const int dx = 2 * tx + fcc_half(bj, 0) - fcc_half(b, 0);
          const int dy = 2 * ty + fcc_half(bj, 1) - fcc_half(b, 1);
          const int dz = 2 * tz + fcc_half(bj, 2) - fcc_half(b, 2);
          if (bj != b && dx * dx + dy * dy + dz * dz == 2) {
            if (n == k) return Slot{tx, ty, tz, bj};
            ++n;
          }
        }
  return Slot{0, 0, 0, -1};
}

struct FamFCC {
  static constexpr int id = kFamFCC, SEP = 0;
  static constexpr int NB = 4, RX = 1, RY = 1, RZ = 1, TWO_D = 0;
  static constexpr int NSHELL = 1, Z = 12, REST = 0;
  __host__ __device__ static constexpr int shell_end(int /*b*/, int /*g*/) { return 12; }
  __host__ __device__ static constexpr Slot slot(int b, int k) { return fcc_shell1(b, k); }
};

// fcc with the second shell: the 6 same-sublattice neighbours at a
struct FamFCC2 {
  static constexpr int id = kFamFCC2, SEP = 0;
  static constexpr int NB = 4, RX = 1, RY = 1, RZ = 1, TWO_D = 0;
  static constexpr int NSHELL = 2, Z = 18, REST = 0;
  __host__ __device__ static constexpr int shell_end(int /*b*/, int g) { return g == 0 ? 12 : 18; }
  __host__ __device__ static constexpr Slot slot(int b, int k) {
    return k < 12 ? fcc_shell1(b, k) : bcc_shell2(b, k - 12);
  }
};

// triangular monolayer (a1, a2 at 60 degrees), 6 neighbours; isotropic part
// as one shell plus a per-slot 3x3 remainder (DMI, anisotropic exchange).
// Tile coordinates (X, Y, Z) = (a1, a3, a2).
struct FamTRI {
  static constexpr int id = kFamTRI, SEP = 0;
  static constexpr int NB = 1, RX = 1, RY = 0, RZ = 1, TWO_D = 1;
  static constexpr int NSHELL = 1, Z = 6, REST = 1;
  __host__ __device__ static constexpr int shell_end(int /*b*/, int /*g*/) { return 6; }
  __host__ __device__ static constexpr Slot slot(int /*b*/, int k) {
    // lattice translations (T1, T2): (1,0) (-1,0) (0,1) (0,-1) (1,-1) (-1,1); dz = T2
    return k == 0 ? Slot{1, 0, 0, 0} : k == 1 ? Slot{-1, 0, 0, 0} : k == 2 ? Slot{0, 0, 1, 0}
         : k == 3 ? Slot{0, 0, -1, 0} : k == 4 ? Slot{1, 0, -1, 0} : Slot{-1, 0, 1, 0};
  }
};

}  // namespace jams_llg
