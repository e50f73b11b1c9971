// The single-precision screen of a trial position against the particles of
// its cell and of the 26 cells around it, as the move pass runs it, shared by
// the move pass (move_pass.cu) and the overlap replay (observables.cu) so
// that a replayed trial is screened with the same arithmetic.
//
// Coordinates are the grid coordinates of the sweep's shifted grid
// (axis_cell): a neighbour seen across a periodic face is shifted by the
// box side L32 (image_of).  A pair whose single-precision r^2 lies below
// lo = 1 - band overlaps, above hi = 1 + band does not, and in between the
// reference's FP64 distance decides (check_overlap / compute_dist,
// src/moves.c:157-212 and 400-431).  The band bounds the single-precision
// error of r^2 with a factor of about two to spare; the derivation is in
// make_box (api.cu).
#pragma once

#include "engine.cuh"

namespace hsmc {

// Neighbour offsets of the 26 cells around a cell, packed (dx+1) | (dy+1)<<2
// | (dz+1)<<4, in the order x-major, the cell itself left out.
__constant__ unsigned char c_nbr[26] = {
    0x00, 0x10, 0x20, 0x04, 0x14, 0x24, 0x08, 0x18, 0x28, 0x01, 0x11, 0x21, 0x05,
    0x25, 0x09, 0x19, 0x29, 0x02, 0x12, 0x22, 0x06, 0x16, 0x26, 0x0a, 0x1a, 0x2a};

// Periodic image (a multiple of the box side) of neighbour `code` of cell
// (ix, iy, iz) as seen from that cell.
__device__ __forceinline__ void image_of(unsigned code, int ix, int iy, int iz, const int *nc, const float *L32,
                                         float &imx, float &imy, float &imz) {
  const int ox = (int)(code & 3u) - 1, oy = (int)((code >> 2) & 3u) - 1, oz = (int)(code >> 4) - 1;
  imx = (ix + ox < 0) ? -L32[0] : (ix + ox >= nc[0] ? L32[0] : 0.f);
  imy = (iy + oy < 0) ? -L32[1] : (iy + oy >= nc[1] ? L32[1] : 0.f);
  imz = (iz + oz < 0) ? -L32[2] : (iz + oz >= nc[2] ? L32[2] : 0.f);
}

// Index of neighbour `code` of cell c = (ix, iy, iz): a linear offset for an
// interior cell, periodic wrapping otherwise.
__device__ __forceinline__ int neighbour_cell(unsigned code, int ix, int iy, int iz, int c, const int *nc,
                                              bool interior) {
  const int ox = (int)(code & 3u) - 1, oy = (int)((code >> 2) & 3u) - 1, oz = (int)(code >> 4) - 1;
  if (interior) return c + ox + nc[0] * (oy + nc[1] * oz);
  int x = ix + ox, y = iy + oy, z = iz + oz;
  x += x < 0 ? nc[0] : (x >= nc[0] ? -nc[0] : 0);
  y += y < 0 ? nc[1] : (y >= nc[1] ? -nc[1] : 0);
  z += z < 0 ? nc[2] : (z >= nc[2] ? -nc[2] : 0);
  return x + nc[0] * (y + nc[1] * z);
}

// Single-precision squared distance of a trial position u from a (possibly
// imaged) neighbour entry q.
__device__ __forceinline__ float dist2(float ux, float uy, float uz, const float4 &q) {
  const float dx = ux - q.x, dy = uy - q.y, dz = uz - q.z;
  return dx * dx + dy * dy + dz * dz;
}

// A neighbour slot as the screen sees it: its grid coordinates plus the
// periodic image, added only when the image is not zero (as the move pass
// adds it to the pool entries of a boundary cell).
__device__ __forceinline__ float4 imaged_entry(const Slot &o, float imx, float imy, float imz) {
  float4 v = make_float4(o.x, o.y, o.z, __int_as_float(o.id));
  if (imx != 0.f || imy != 0.f || imz != 0.f) {
    v.x = __fadd_rn(v.x, imx);
    v.y = __fadd_rn(v.y, imy);
    v.z = __fadd_rn(v.z, imz);
  }
  return v;
}

}  // namespace hsmc
