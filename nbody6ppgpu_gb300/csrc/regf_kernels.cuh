// Regular force + jerk + potential + neighbour list kernels (sm_103a).
//
// Replaces the device side of src/Main/gpunb.velocity.cu:162-552
// (dev_gravity / gravity_kernel / force_reduce_kernel / gather_nb_kernel).
#pragma once
#include "common.cuh"

namespace gpunb {

// ---------------------------------------------------------------------------
// j-tile layout (split precision).  JT bodies per tile, SoA fields, then one
// float4 of tile metadata.  One tile is one 16-byte-aligned bulk copy.
constexpr int JT = 128;
enum JField { F_XH = 0, F_YH, F_ZH, F_XL, F_YL, F_ZL, F_VX, F_VY, F_VZ, F_MN, NFIELD };
constexpr int TILE_FLOATS = NFIELD * JT + 4;
constexpr int TILE_BYTES = TILE_FLOATS * 4;
static_assert(TILE_BYTES % 16 == 0, "tile must be a multiple of 16 bytes");
// F_MN holds -m/2: the force loop forms -2/r in its Newton step, so that
// (-m/2)*(-2/r) = m/r needs no negation.
// metadata: [0] = max |v_j| over the tile (rounded up), [1] = sqrt(max m_j)
// (rounded up), [2] = number of real bodies in the tile, [3] unused.

// FP64 j tile for the plain FP64 kernel (three bulk copies per tile).
constexpr int JT64 = 64;

// Number of partial quantities per i: ax ay az jx jy jz pot.
constexpr int NQ = 7;

struct JSet {
  const float *tiles;    // [ntile][TILE_FLOATS]
  const double *m64;     // [nj]
  const double *x64;     // [nj][3]
  const double *v64;     // [nj][3]
  const int *perm;       // tile slot -> index into the sent arrays (Morton order)
  int nj;
  int ntile;             // ceil(nj / JT)
  int ntile64;           // ceil(nj / JT64)
};

struct ISet {
  const double *h2;      // [ni]
  const double *dtr;     // [ni]
  const double *x;       // [ni][3]
  const double *v;       // [ni][3]
  const int *perm;       // processing slot -> i index (Morton order), or null
  const float4 *rec;     // [ni][4] FP32 i-records in slot order (regf_prep_kernel)
  int ni;
};

// One work item of the pair kernel: an i-tile against a range of j tiles.
// Partial sums of slot s go to part[(prow*NQ + q)*ni_pad + pcol0 + (s - slot0)].
struct ItemDesc {
  int slot0;      // first processing slot of the i-tile
  int slot_end;   // end of the owning j-set's slots (exclusive)
  int t0, t1;     // tile range [t0, t1)
  int prow;       // partial-sum row
  int jbase;      // first index of the owning j-set (reported ids are relative)
  int pcol0;      // partial-sum column of slot0
  int pad;
};

struct RegfOut {
  double *part;          // [rows][NQ][ni_pad] partial sums, column = processing slot
  int *cnt;              // [ni] neighbour counters (zeroed before the launch)
  int *rows;             // [ni][cap] unsorted neighbour ids
  int cap;               // row capacity (= nnbmax)
  int ni_pad;
  int *err;              // device error word
};

}  // namespace gpunb
