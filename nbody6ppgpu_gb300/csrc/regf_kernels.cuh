// Regular force + jerk + potential + neighbour list kernels (sm_103a).
//
// Replaces the device side of src/Main/gpunb.velocity.cu:162-552
// (dev_gravity / gravity_kernel / force_reduce_kernel / gather_nb_kernel).
#pragma once
#include "common.cuh"

namespace gpunb {

// ---------------------------------------------------------------------------
// j-tile layout.  JT bodies per tile (consecutive along the Morton curve),
// SoA fields, then three float4 of tile metadata.  One tile is one
// 16-byte-aligned bulk copy.  Positions are held twice:
//   * relative to the tile's centre O (the midpoint of its bounding box) as
//     single FP32 values.  A thread forms, once per tile, the offset
//     o = O - x_i of its i-particle in double-single arithmetic rounded to
//     FP32, and per pair dx = (x_j - O) + o: one addition per component.
//     The rounding of x_j - O is at most 2^-24 of the tile radius R, so dx
//     carries an absolute error below 2^-22 (R + |dx|) per component, within
//     2^-21 |dx| for the tiles this path is used for (|o| >= 2R);
//   * as double-single hi/lo pairs, for the tiles near the warp's i-particles
//     (for one of them |o| < 2R and R + |o| > 3 d, d the distance to the
//     tile's box): dx = (hi_j - hi_i) + (lo_j - lo_i), three additions per
//     component, error 2^-23 |dx|.
#ifndef GPUNB_JT
#define GPUNB_JT 128
#endif
constexpr int JT = GPUNB_JT;
static_assert(JT % 64 == 0 && JT <= 1024, "a tile holds a multiple of 64 bodies");
enum JField {
  F_XR = 0, F_YR, F_ZR, F_VX, F_VY, F_VZ, F_MN,   // far tiles read these 7
  F_XH, F_YH, F_ZH, F_XL, F_YL, F_ZL,             // near tiles: velocity, mass and these
  NFIELD
};
constexpr int NFIELD_REL = F_MN + 1;
constexpr int TILE_META = 12;
constexpr int TILE_FLOATS = NFIELD * JT + TILE_META;
constexpr int TILE_BYTES = TILE_FLOATS * 4;
static_assert(TILE_BYTES % 16 == 0, "tile must be a multiple of 16 bytes");
// F_MN holds -m/2: the force loop forms -2/r in its Newton step, so that
// (-m/2)*(-2/r) = m/r needs no negation.
// metadata (float offsets from NFIELD*JT):
//   [0] max |v_j| over the tile (rounded up)   [1] sqrt(max m_j) (rounded up)
//   [2] number of real bodies                  [3] tile radius R (rounded up)
//   [4..6] O (x, y, z), an FP32 number          [7] unused
//   [8..10] half-extents of the tile's box      [11] unused
enum TileMeta { M_VMAX = 0, M_SMAX, M_COUNT, M_RAD, M_OH = 4, M_BOX = 8 };

// A tile is "near" an i-particle, and its pairs take the double-single
// coordinate path, when |O - x_i|^2 < GPUNB_NEAR_K2 R^2.  With K = 2 every
// pair of a far tile is at least R away, so the tile-relative rounding
// (2^-22 (R + |dx|) per axis) stays within 2^-21 |dx|.  Measured against the
// FP64 kernel (Plummer 65536 and King 2^20, ni = 16384): force and jerk
// errors equal to the all-double-single kernel's to two digits, while
// K = 0 (every tile relative) doubled the jerk's 99th percentile; the pair
// kernel gains 7% (N = 65536) to 13% (N = 2^20) over K = infinity.
#ifndef GPUNB_NEAR_K2
#define GPUNB_NEAR_K2 4.0f
#endif

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
  // Merge in the pair kernel (single j-set, split kernel; done == null: a
  // merge kernel follows): the block that completes the last of an i-tile's
  // S items sums the tile's partial rows in split order and stores the
  // results as the merge kernels do.
  int *done = nullptr;   // [n_itiles] completed items per i-tile (zeroed before the launch)
  const int *perm = nullptr;   // processing slot -> i (null: identity)
  double *acc = nullptr, *jrk = nullptr, *pot = nullptr;
  int *nnb = nullptr, *rowlen = nullptr;
  int nnbmax = 0;
};

}  // namespace gpunb
