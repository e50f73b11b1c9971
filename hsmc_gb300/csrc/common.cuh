// Device-side building blocks shared by the GB300 hard-sphere kernels:
// counter-based random numbers, the reference's FP64 distance arithmetic,
// the shifted periodic cell grid, and the device-resident state structs.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cavity_coeffs.h"

namespace hsmc {

// ---------------------------------------------------------------- Philox
// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64 multiplies, with the
// 64-bit key bumped by the Weyl constants between rounds.
struct U32x4 {
  uint32_t x, y, z, w;
};

__host__ __device__ inline void mul_hilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

__host__ __device__ inline U32x4 philox4x32_10(U32x4 c, uint32_t k0, uint32_t k1) {
  const uint32_t m0 = 0xD2511F53u, m1 = 0xCD9E8D57u;
  const uint32_t w0 = 0x9E3779B9u, w1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t h0, l0, h1, l1;
    mul_hilo(m0, c.x, h0, l0);
    mul_hilo(m1, c.z, h1, l1);
    c = U32x4{h1 ^ c.y ^ k0, l1, h0 ^ c.w ^ k1, l0};
    k0 += w0;
    k1 += w1;
  }
  return c;
}

// Counter spaces: the top four bits of the last counter word name the use,
// so streams for different purposes never share a counter.
enum : uint32_t {
  TAG_MOVE = 1u,
  TAG_SHIFT = 2u,
  TAG_PERM = 3u,
  TAG_WIDOM = 4u,
  TAG_VOLUME = 5u,
  TAG_CLUSTER = 7u,  // 6 is the learned Widom sampler's
  TAG_CAVITY = 8u,
};

__host__ __device__ inline U32x4 draw4(uint64_t seed, uint32_t a, uint32_t b, uint64_t seq, uint32_t tag) {
  U32x4 c{a, b, (uint32_t)seq, (tag << 28) | ((uint32_t)(seq >> 32) & 0x0fffffffu)};
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// Exact dyadic numbers built from a 32-bit draw with integer operations only
// (GB300 has a narrow FP64 pipe; none of this touches it).
//   centred_offset(r) = (2r - 2^32 + 1) * 2^-33, odd multiples of 2^-33 in
//                       (-1/2, 1/2), symmetric about 0: the trial step factor
//                       (u - 0.5) of part_move (src/moves.c:52-54)
//   open_unit(r)      = (2r + 1) * 2^-33 in (0, 1): the uniform of
//                       widom_rand_pos and vol_move (src/compute_widom_chem_pot.c:76-78,
//                       src/moves.c:91)
// The reference draws u = r / (2^32 - 1) in [0, 1]; the same u is obtained
// from the reference's own code with a generator maximum of 2^33 and the
// draw 2r + 1, which is how the replay harness feeds it.
__device__ __forceinline__ double dyadic_2m33(uint64_t mag, bool neg) {
  // mag in [1, 2^33): value = mag * 2^-33, exactly representable
  const int p = 63 - __clzll((long long)mag);              // leading bit, 0..32
  const uint64_t mant = (mag << (52 - p)) & 0x000FFFFFFFFFFFFFull;
  const uint64_t expo = (uint64_t)(p - 33 + 1023);
  return __longlong_as_double((long long)(((uint64_t)neg << 63) | (expo << 52) | mant));
}

__device__ __forceinline__ double centred_offset(uint32_t r) {
  const long long v = 2ll * (long long)r - 4294967295ll;  // odd, |v| < 2^32
  return dyadic_2m33((uint64_t)(v < 0 ? -v : v), v < 0);
}

__device__ __forceinline__ double open_unit(uint32_t r) { return dyadic_2m33(2ull * r + 1ull, false); }

// x < y for doubles by their bit patterns when y > 0 is finite: negative x
// (sign bit set, not -0.0) is below; otherwise the patterns order as integers.
__device__ __forceinline__ bool gt_pos(double x, double y) {
  const long long a = __double_as_longlong(x), b = __double_as_longlong(y);
  return a > b;  // x with sign bit set is a negative integer pattern: never > b > 0
}

__device__ __forceinline__ bool lt_zero(double x) {
  const long long a = __double_as_longlong(x);
  return a < 0 && (a & 0x7FFFFFFFFFFFFFFFll) != 0;  // -0.0 is not below zero
}

// ------------------------------------------------- reference arithmetic
// Trial position x + (u - 0.5) * dr_max with no contraction
// (src/moves.c:52-54), t = u - 0.5 given exactly, then the single periodic
// wrap of apply_pbc (src/moves.c:215-226) with the comparisons done on bit
// patterns: two FP64 operations per axis on the common path.
__device__ __forceinline__ double propose_axis(double x, double t, double dr_max, double len) {
  double v = __dadd_rn(x, __dmul_rn(t, dr_max));
  if (gt_pos(v, len)) v = __dsub_rn(v, len);
  else if (lt_zero(v)) v = __dadd_rn(v, len);
  return v;
}

// One component of compute_dist (src/moves.c:413-424) with sf = 1:
// difference, then one minimum-image branch.
__device__ __forceinline__ double min_image(double d, double len, double half) {
  if (d > half) d = __dsub_rn(d, len);
  else if (d < -half) d = __dadd_rn(d, len);
  return d;
}

// Squared distance in the reference's order ((dx*dx + dy*dy) + dz*dz), no
// FMA.  sqrt is correctly rounded and monotone, so sqrt(r2) < 1 exactly when
// r2 < 1: the reference's overlap decision is r2 < 1.0.
__device__ __forceinline__ double ref_r2(double ax, double ay, double az, double bx, double by, double bz,
                                         const double *len, const double *half) {
  double dx = min_image(__dsub_rn(ax, bx), len[0], half[0]);
  double dy = min_image(__dsub_rn(ay, by), len[1], half[1]);
  double dz = min_image(__dsub_rn(az, bz), len[2], half[2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Scaled form used by the volume move and the thermodynamic pressure
// (compute_dist with sf < 1, src/moves.c:400-431): dx = (a - b) * sf, box
// side L * sf, half side (L * sf) / 2.
__device__ __forceinline__ double ref_r2_scaled(double ax, double ay, double az, double bx, double by, double bz,
                                                const double *len, double sf) {
  double lx = __dmul_rn(len[0], sf), ly = __dmul_rn(len[1], sf), lz = __dmul_rn(len[2], sf);
  double dx = min_image(__dmul_rn(__dsub_rn(ax, bx), sf), lx, lx * 0.5);
  double dy = min_image(__dmul_rn(__dsub_rn(ay, by), sf), ly, ly * 0.5);
  double dz = min_image(__dmul_rn(__dsub_rn(az, bz), sf), lz, lz * 0.5);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// ---------------------------------------------------------- cell grid
// Positions are binned on a periodic grid of nc (even) cells per axis,
// shifted by s in [0, w).  t = x32 - s (wrapped into [0, L)) is the
// coordinate along the shifted grid; cell = floor(t / w).  The same
// single-precision arithmetic assigns particles at build time and confines
// moves, so membership is always self-consistent; the cell edge carries a
// margin over 1 that absorbs the rounding of x32 and t.
__device__ __forceinline__ void axis_cell(float x32, float s32, float len32, float inv_w32, int nc, int &cell,
                                          float &t) {
  t = __fsub_rn(x32, s32);
  if (t < 0.0f) t = __fadd_rn(t, len32);
  cell = (int)__fmul_rn(t, inv_w32);
  if (cell >= nc) {
    cell -= nc;
    t = __fsub_rn(t, len32);
  }
}

// ------------------------------------------------------- device state
struct Box {
  double len[3];      // box sides L
  double half[3];     // L / 2.0
  double vol, rho;
  float len32[3];     // (float)L
  float inv_w32[3];   // (float)(nc / L)
  float w32[3];       // (float)(L / nc), scale of the grid shift
  float band;         // half-width of the single-precision screen on r^2
  int nc[3];          // cells per axis (even, >= 4)
  int ncell;
  int pad;
};

struct SweepParams {
  unsigned long long sweep;  // global index of the sweep whose layout is current
  float shift32[3];          // grid shift of that sweep
  int perm[8];               // colour order of its eight passes
};

// Status bits set by kernels (the host maps them to hsmc_status codes).
enum : int {
  ST_CELL_OVERFLOW = 1,
  ST_BAD_BIN = 2,
  ST_OUT_OF_BOX = 4,
  ST_TRACE_FULL = 8,
  ST_BAD_CELL = 16,
  ST_FLOW_TIMEOUT = 32,     // a dataflow wait gave up (the sweep's result is invalid)
  ST_CLUSTER_TIMEOUT = 64,  // a cluster move's grid-wide wait gave up (its result is invalid)
  ST_CAVITY_RANGE = 128,    // the cavities' distance was outside the allowed range before a cavity move
  ST_BAD_ID = 256,          // an uploaded configuration's id column is not 0, 1, ..., N - 1
};

struct DevState {
  unsigned long long sweep_base;  // index of the next sweep to run
  unsigned long long acc;         // accepted particle moves
  unsigned long long rej_overlap;
  unsigned long long rej_boundary;
  unsigned long long rechecks;    // pairs re-evaluated in FP64
  unsigned long long vol_moves, vol_acc;
  unsigned long long trace_count;
  unsigned long long widom_ok;
  unsigned long long scan_mask[4];  // thermodynamic-pressure overlap bits
  unsigned long long cav_moves, cav_acc;  // cavity trials and acceptances
  double dr_max, dv_max, pressure;
  unsigned long long seed;
  unsigned long long cav_trace_count;  // cavity-trial records since the last read
  int status;
  int pad;
  SweepParams params;
  // NpT: the trial volume move of the current sweep and the lattice the box
  // is rebuilt from (sim_box_init, src/sim_info.c:32-71)
  double vol_sf, vol_new, vol_ratio, vol_u_acc;
  int vol_overlap, vol_accept;
  int cells[3], per_cell;
  int nc_alloc[3];
  int flow_hold;  // dataflow schedule: a region that does not publish (diagnostic), -1 for none
  // cavity sampling: particles below `frozen` (the two cavities) are left in
  // place by the colour passes and moved by k_cavity, cav_trials per sweep
  int frozen;
  int cav_trials;
  double cav_min, cav_max;
  // sqrt(r2) >= cav_min exactly when r2 >= cav_r2min, and sqrt(r2) <= cav_max
  // exactly when r2 <= cav_r2max (sqrt is correctly rounded, so monotone)
  double cav_r2min, cav_r2max;
  hsmc_cavity_psi_coeffs psi;
  // the device optimiser (hsmc_gpu_optimize): the secant's last two points
  // (step, acceptance) for the particle and the volume step, and the counters
  // at the start of the current sample
  double opt_d[2], opt_a[2], opt_v[2], opt_av[2];
  unsigned long long opt_acc0, opt_moves0, opt_vacc0, opt_vmoves0;
};

// One particle in a cell: its grid coordinates t (single precision, from
// axis_cell of the rounded position, so t lies in the cell's own slab of
// [0, L)) and its id.
struct alignas(16) Slot {
  float x, y, z;
  int id;
};

// Colour (0..7) of a cell of the 2x2x2 checkerboard.
__host__ __device__ __forceinline__ int cell_colour(int ix, int iy, int iz) {
  return (ix & 1) | ((iy & 1) << 1) | ((iz & 1) << 2);
}

// FP64 coordinates of particle id from the double[N][4] (id, x, y, z) array:
// two aligned 16-byte loads.
__device__ __forceinline__ void load_xyz(const double *pos, int id, double &x, double &y, double &z) {
  const double2 a = *reinterpret_cast<const double2 *>(pos + 4 * (size_t)id);
  const double2 b = *reinterpret_cast<const double2 *>(pos + 4 * (size_t)id + 2);
  x = a.y;
  y = b.x;
  z = b.y;
}

// Counters of one launch reduced per warp, then added once per warp.
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace hsmc
