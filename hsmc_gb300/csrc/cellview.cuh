// Read-only view of the current cell layout for kernels that sample
// observables or test insertions between sweeps (observables.cu, lwidom.cu).
#pragma once

#include "engine.cuh"

namespace hsmc {

struct Stencil {
  int k[3];  // half-width in cells per axis; -1 means every cell of the axis
};

struct CellView {
  const int *cnt;
  const Slot *slot;
  int cap;
  int nc[3];
  float sh[3], L32[3], iw[3], w[3];
  float band;  // the move pass's guard band on r^2 (the box's)
};

// Squared distance, less a margin, from a particle at grid coordinate t in
// cell ci to the nearest point of the cell o cells away along an axis: a
// cell of a stencil whose nearest point is beyond the cut holds no pair
// within it and is not read.  Cell faces lie at multiples of w = L / nc up to
// the rounding of the cell assignment; the margin (1e-3, far above that
// rounding) keeps the test conservative.
struct StencilGap {
  float lo[3] = {0.f, 0.f, 0.f}, hi[3] = {0.f, 0.f, 0.f}, w[3] = {0.f, 0.f, 0.f};

  __device__ __forceinline__ void init(const int ci[3], const float t[3], const float w32[3]) {
    for (int d = 0; d < 3; d++) {
      w[d] = w32[d];
      lo[d] = t[d] - (float)ci[d] * w32[d];        // to the cell's lower face
      hi[d] = (float)(ci[d] + 1) * w32[d] - t[d];  // to its upper face
    }
  }
  __device__ __forceinline__ float sq(int d, int o) const {
    if (o == 0) return 0.f;
    const float g = (o > 0 ? hi[d] + (float)(o - 1) * w[d] : lo[d] + (float)(-o - 1) * w[d]) - 1e-3f;
    return g > 0.f ? g * g : 0.f;
  }
};

__device__ __forceinline__ CellView current_view(const SysPtrs &p) {
  CellView v;
  const DevState *st = p.st;
  const Box *bx = p.box;
  const int layout = (int)(st->params.sweep & 1ull);
  v.cnt = cnt_of(p, layout);
  v.slot = slot_of(p, layout);
  v.cap = p.cap;
  for (int d = 0; d < 3; d++) {
    v.nc[d] = bx->nc[d];
    v.sh[d] = st->params.shift32[d];
    v.L32[d] = bx->len32[d];
    v.iw[d] = bx->inv_w32[d];
    v.w[d] = bx->w32[d];
  }
  v.band = bx->band;
  return v;
}

// Visit the particles in the stencil of the cell holding (x, y, z), cell by
// cell in a fixed order, until visit returns true.  With PRUNE, cells whose
// nearest point lies beyond sqrt(cut2) are skipped (an axis that spans every
// cell is not pruned); the thermodynamic scan, whose stencil is the 27
// cells, measured faster without (the test costs it registers).
template <bool PRUNE = true, class F>
__device__ __forceinline__ void for_each_near(const CellView &v, const Stencil &s, double x, double y, double z,
                                              float cut2, F &&visit) {
  int ci[3];
  float t[3];
  axis_cell(__double2float_rn(x), v.sh[0], v.L32[0], v.iw[0], v.nc[0], ci[0], t[0]);
  axis_cell(__double2float_rn(y), v.sh[1], v.L32[1], v.iw[1], v.nc[1], ci[1], t[1]);
  axis_cell(__double2float_rn(z), v.sh[2], v.L32[2], v.iw[2], v.nc[2], ci[2], t[2]);
  StencilGap gap;
  if (PRUNE) gap.init(ci, t, v.w);
  int lo[3], span[3];
  for (int d = 0; d < 3; d++) {
    if (s.k[d] < 0) {
      lo[d] = 0;
      span[d] = v.nc[d];
    } else {
      lo[d] = ci[d] - s.k[d];
      span[d] = 2 * s.k[d] + 1;
    }
  }
  for (int a = 0; a < span[2]; a++) {
    const float gz = (!PRUNE || s.k[2] < 0) ? 0.f : gap.sq(2, a - s.k[2]);
    if (gz > cut2) continue;
    int cz = lo[2] + a;
    cz = (cz % v.nc[2] + v.nc[2]) % v.nc[2];
    for (int b = 0; b < span[1]; b++) {
      const float gzy = gz + ((!PRUNE || s.k[1] < 0) ? 0.f : gap.sq(1, b - s.k[1]));
      if (gzy > cut2) continue;
      int cy = lo[1] + b;
      cy = (cy % v.nc[1] + v.nc[1]) % v.nc[1];
      for (int e = 0; e < span[0]; e++) {
        if (PRUNE && gzy + (s.k[0] < 0 ? 0.f : gap.sq(0, e - s.k[0])) > cut2) continue;
        int cx = lo[0] + e;
        cx = (cx % v.nc[0] + v.nc[0]) % v.nc[0];
        const int c = cx + v.nc[0] * (cy + v.nc[1] * cz);
        const int m = v.cnt[c];
        const int n = m < v.cap ? m : v.cap;  // an overfull cell was flagged by the build
        const Slot *sl = v.slot + (size_t)c * v.cap;
        for (int q = 0; q < n; q++)
          if (visit(sl[q])) return;
      }
    }
  }
}

// Grid coordinates of a point (the slots hold particles this way).
__device__ __forceinline__ void grid_coords(const CellView &v, double x, double y, double z, float &tx, float &ty,
                                            float &tz) {
  int ci;
  axis_cell(__double2float_rn(x), v.sh[0], v.L32[0], v.iw[0], v.nc[0], ci, tx);
  axis_cell(__double2float_rn(y), v.sh[1], v.L32[1], v.iw[1], v.nc[1], ci, ty);
  axis_cell(__double2float_rn(z), v.sh[2], v.L32[2], v.iw[2], v.nc[2], ci, tz);
}

// Single-precision squared minimum-image distance, for discarding far pairs.
__device__ __forceinline__ float approx_r2(float ax, float ay, float az, const Slot &o, const float *L32) {
  float dx = ax - o.x, dy = ay - o.y, dz = az - o.z;
  dx -= L32[0] * rintf(dx / L32[0]);
  dy -= L32[1] * rintf(dy / L32[1]);
  dz -= L32[2] * rintf(dz / L32[2]);
  return dx * dx + dy * dy + dz * dz;
}

// widom_rand_pos (src/compute_widom_chem_pot.c:73-80): x = u * L with u the
// reference's closed uniform; widom_compute_dist (:130-160): insertion minus
// particle, one minimum-image branch, overlap when r < 1.  The
// single-precision r^2 decides outside the guard band of contact (its error
// is below the band, as in the move pass's screen: the minimum-image shift
// here is an exact subtraction of the box side); inside it the reference's
// FP64 distance decides.
__device__ __forceinline__ bool point_overlaps(const CellView &v, const SysPtrs &p, const Stencil &s, double x,
                                               double y, double z, int skip, const double *len,
                                               const double *half) {
  float x32, y32, z32;  // grid coordinates, as the slots hold them
  grid_coords(v, x, y, z, x32, y32, z32);
  const float lo = 1.0f - v.band, hi = 1.0f + v.band;
  bool ov = false;
  for_each_near(v, s, x, y, z, hi, [&](const Slot &o) {
    if (o.id == skip) return false;
    const float r2 = approx_r2(x32, y32, z32, o, v.L32);
    if (r2 < lo) {
      ov = true;
      return true;
    }
    if (r2 > hi) return false;
    double ox, oy, oz;
    load_xyz(p.pos, o.id, ox, oy, oz);
    if (ref_r2(x, y, z, ox, oy, oz, len, half) < 1.0) ov = true;
    return ov;
  });
  return ov;
}

}  // namespace hsmc
