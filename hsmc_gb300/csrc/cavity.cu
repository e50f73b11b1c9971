// Cavity sampling (cavity_part_move / cavity_check_move, src/moves.c:254-396)
// on the device: the cavity stage of each sweep of a cavity run.
//
// Particles 0 and 1 are the two cavities.  The colour passes leave them in
// place (move_pass.cu, DevState::frozen); after the passes of a sweep one warp
// makes the sweep's cavity trials one after the other, because each depends
// on where the previous one left the pair:
//   - a cavity (one bit of the draw) is displaced as in part_move;
//   - the move is rejected when the new distance between the cavities leaves
//     [cav_min, cav_max], or by the Metropolis test on the umbrella potential
//     psi = ln y_GH against a uniform, or when the moved cavity overlaps a
//     particle other than the cavities (lane k of the warp tests neighbour
//     cell k of the 27, single precision outside the guard band, the
//     reference's FP64 distance inside it).
// The other particles do not move during the stage, so the sweep's cell
// layout still holds them; the cavities' own entries in it are not used.
#include "cavity.cuh"
#include "cellview.cuh"

namespace hsmc {

namespace {

__global__ void k_cavity_psi(const DevState *st, const double *x, int n, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cavity_psi(st->psi, x[i]);
}

// The cavity trials of sweep sweep_base + offset (one warp), screening the
// sweep's cell layout: lane k tests neighbour cell k of the 27.
__global__ void __launch_bounds__(32) k_cavity(SysPtrs p, long long offset, uint32_t *trace, long long trace_cap) {
  DevState *st = p.st;
  const unsigned long long s = st->sweep_base + (unsigned long long)offset;
  const CellView v = current_view(p);
  const Box *bx = p.box;
  double len[3], half[3];
  for (int d = 0; d < 3; d++) {
    len[d] = bx->len[d];
    half[d] = bx->half[d];
  }
  const float band = bx->band;
  const int lane = (int)threadIdx.x;
  const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
  double cav[2][3];
  for (int w = 0; w < 2; w++) load_xyz(p.pos, w, cav[w][0], cav[w][1], cav[w][2]);
  auto overlaps = [&](const double *nw) -> bool {
    bool ov = false;
    if (lane < 27) {
      int ci[3];
      float t[3];
      axis_cell(__double2float_rn(nw[0]), v.sh[0], v.L32[0], v.iw[0], v.nc[0], ci[0], t[0]);
      axis_cell(__double2float_rn(nw[1]), v.sh[1], v.L32[1], v.iw[1], v.nc[1], ci[1], t[1]);
      axis_cell(__double2float_rn(nw[2]), v.sh[2], v.L32[2], v.iw[2], v.nc[2], ci[2], t[2]);
      int cx = ci[0] + ox, cy = ci[1] + oy, cz = ci[2] + oz;
      cx = cx < 0 ? cx + v.nc[0] : (cx >= v.nc[0] ? cx - v.nc[0] : cx);
      cy = cy < 0 ? cy + v.nc[1] : (cy >= v.nc[1] ? cy - v.nc[1] : cy);
      cz = cz < 0 ? cz + v.nc[2] : (cz >= v.nc[2] ? cz - v.nc[2] : cz);
      const int c = cx + v.nc[0] * (cy + v.nc[1] * cz);
      const int m = v.cnt[c];
      const int nq = m < v.cap ? m : v.cap;
      const Slot *sl = v.slot + (size_t)c * v.cap;
      for (int q = 0; q < nq && !ov; q++) {
        const Slot o = sl[q];
        if (o.id < 2) continue;  // the cavities do not overlap each other
        const float r2f = approx_r2(t[0], t[1], t[2], o, v.L32);
        if (r2f > 1.0f + band) continue;
        if (r2f < 1.0f - band) {
          ov = true;
        } else {
          double px, py, pz;
          load_xyz(p.pos, o.id, px, py, pz);
          ov = ref_r2(nw[0], nw[1], nw[2], px, py, pz, len, half) < 1.0;
        }
      }
    }
    return __any_sync(0xffffffffu, ov);
  };
  auto accept = [&](int w, const double *nw) {
    if (lane == 0) {
      double *q = p.pos + 4 * (size_t)w;
      q[1] = nw[0];
      q[2] = nw[1];
      q[3] = nw[2];
    }
  };
  unsigned long long done = 0, acc = 0;
  cavity_trials(st, s, cav, len, half, overlaps, accept, trace, trace_cap, &st->cav_trace_count, &st->status, done,
                acc);
  if (lane == 0) {
    atomicAdd(&st->cav_moves, done);
    atomicAdd(&st->cav_acc, acc);
  }
}

}  // namespace

void launch_cavity(const SysPtrs &p, long long sweep_offset, uint32_t *trace, long long trace_cap,
                   cudaStream_t s) {
  k_cavity<<<1, 32, 0, s>>>(p, sweep_offset, trace, trace_cap);
}

void launch_cavity_psi(const SysPtrs &p, const double *x, int n, double *out, cudaStream_t s) {
  if (n > 0) k_cavity_psi<<<(n + 127) / 128, 128, 0, s>>>(p.st, x, n, out);
}

}  // namespace hsmc
