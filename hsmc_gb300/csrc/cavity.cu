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
#include "cellview.cuh"

namespace hsmc {

namespace {

// psi(x) = lny_gh(x, pi rho / 6, 1) (src/analytic.c:34-54): the
// Grundke-Henderson cubic inside the core, ln g_VW outside, with g_VW the
// Percus-Yevick g at x / dW plus a damped oscillation (rdf_vw and rdf_py,
// src/analytic.c:79-99, 143-170), in the reference's operation order.
__device__ double cavity_psi(const hsmc_cavity_psi_coeffs &c, double x) {
  if (x < 1.0) {
    return __dadd_rn(__dadd_rn(__dadd_rn(c.ay[0], __dmul_rn(c.ay[1], x)), __dmul_rn(__dmul_rn(c.ay[2], x), x)),
                     __dmul_rn(__dmul_rn(__dmul_rn(c.ay[3], x), x), x));
  }
  const double d = __dsub_rn(x, 1.0);
  const double osc =
      __dmul_rn(__dmul_rn(__ddiv_rn(c.AA, x), exp(__dmul_rn(-c.mu, d))), cos(__dmul_rn(c.mu, d)));
  // Re sum_k a_k exp(t_k (x / dW - 1)), divided by x / dW
  const double xh = __ddiv_rn(x, c.dW);
  const double dh = __dsub_rn(xh, 1.0);
  double re = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double mag = exp(__dmul_rn(c.t_re[k], dh));
    double sn, cs;
    sincos(__dmul_rn(c.t_im[k], dh), &sn, &cs);
    const double er = __dmul_rn(mag, cs), ei = __dmul_rn(mag, sn);
    const double term = __dsub_rn(__dmul_rn(c.a_re[k], er), __dmul_rn(c.a_im[k], ei));
    re = k == 0 ? term : __dadd_rn(re, term);
  }
  const double g_py = __ddiv_rn(re, xh);
  return log(__dadd_rn(g_py, osc));
}

// The same psi for a warp-uniform x, with the three Percus-Yevick terms and
// the damped oscillation on lanes 0-3 at once (the serial cavity stage waits
// on this latency); every lane returns the value.
__device__ double cavity_psi_warp(const hsmc_cavity_psi_coeffs &c, double x, int lane) {
  if (x < 1.0) {
    return __dadd_rn(__dadd_rn(__dadd_rn(c.ay[0], __dmul_rn(c.ay[1], x)), __dmul_rn(__dmul_rn(c.ay[2], x), x)),
                     __dmul_rn(__dmul_rn(__dmul_rn(c.ay[3], x), x), x));
  }
  const double xh = __ddiv_rn(x, c.dW);
  double part = 0.0;
  if (lane < 3) {
    const double dh = __dsub_rn(xh, 1.0);
    const double mag = exp(__dmul_rn(c.t_re[lane], dh));
    double sn, cs;
    sincos(__dmul_rn(c.t_im[lane], dh), &sn, &cs);
    part = __dsub_rn(__dmul_rn(c.a_re[lane], __dmul_rn(mag, cs)), __dmul_rn(c.a_im[lane], __dmul_rn(mag, sn)));
  } else if (lane == 3) {
    const double d = __dsub_rn(x, 1.0);
    part = __dmul_rn(__dmul_rn(__ddiv_rn(c.AA, x), exp(__dmul_rn(-c.mu, d))), cos(__dmul_rn(c.mu, d)));
  }
  const double t0 = __shfl_sync(0xffffffffu, part, 0), t1 = __shfl_sync(0xffffffffu, part, 1);
  const double t2 = __shfl_sync(0xffffffffu, part, 2), osc = __shfl_sync(0xffffffffu, part, 3);
  return log(__dadd_rn(__ddiv_rn(__dadd_rn(__dadd_rn(t0, t1), t2), xh), osc));
}

// psi in single precision from single-precision coefficients, for deciding
// the Metropolis test away from its edge: its error on psi' - psi is below
// 1e-5 for the densities of a hard-sphere fluid, far inside the 1e-3 band
// the stage leaves to the FP64 value.
struct Psi32 {
  float ay[4], AA, mu, dW, t_re[3], t_im[3], a_re[3], a_im[3];
};

__device__ Psi32 psi32_coeffs(const hsmc_cavity_psi_coeffs &c) {
  Psi32 f;
  for (int k = 0; k < 4; k++) f.ay[k] = (float)c.ay[k];
  f.AA = (float)c.AA;
  f.mu = (float)c.mu;
  f.dW = (float)c.dW;
  for (int k = 0; k < 3; k++) {
    f.t_re[k] = (float)c.t_re[k];
    f.t_im[k] = (float)c.t_im[k];
    f.a_re[k] = (float)c.a_re[k];
    f.a_im[k] = (float)c.a_im[k];
  }
  return f;
}

// For a warp-uniform x; the three Percus-Yevick terms and the oscillation
// on lanes 0-3 at once, every lane returns the value.
__device__ float cavity_psi32(const Psi32 &c, float x, int lane) {
  if (x < 1.0f) return c.ay[0] + x * (c.ay[1] + x * (c.ay[2] + x * c.ay[3]));
  const float xh = x / c.dW, dh = xh - 1.0f;
  float part = 0.0f;
  if (lane < 3) {
    float sn, cs;
    sincosf(c.t_im[lane] * dh, &sn, &cs);
    const float mag = expf(c.t_re[lane] * dh);
    part = c.a_re[lane] * mag * cs - c.a_im[lane] * mag * sn;
  } else if (lane == 3) {
    const float d = x - 1.0f;
    part = (c.AA / x) * expf(-c.mu * d) * cosf(c.mu * d);
  }
  const float re = __shfl_sync(0xffffffffu, part, 0) + __shfl_sync(0xffffffffu, part, 1) +
                   __shfl_sync(0xffffffffu, part, 2);
  return logf(re / xh + __shfl_sync(0xffffffffu, part, 3));
}

__global__ void k_cavity_psi(const DevState *st, const double *x, int n, double *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = cavity_psi(st->psi, x[i]);
}

// The cavity trials of sweep sweep_base + offset (one warp).
__global__ void __launch_bounds__(32) k_cavity(SysPtrs p, long long offset, uint32_t *trace, long long trace_cap) {
  DevState *st = p.st;
  const int trials = st->cav_trials;
  const unsigned long long s = st->sweep_base + (unsigned long long)offset;
  const unsigned long long seed = st->seed;
  const CellView v = current_view(p);
  const Box *bx = p.box;
  double len[3], half[3];
  for (int d = 0; d < 3; d++) {
    len[d] = bx->len[d];
    half[d] = bx->half[d];
  }
  const float band = bx->band;
  const double dr = st->dr_max, cmin = st->cav_min, cmax = st->cav_max;
  const int lane = (int)threadIdx.x;
  const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
  double cav[2][3];
  for (int w = 0; w < 2; w++) load_xyz(p.pos, w, cav[w][0], cav[w][1], cav[w][2]);
  unsigned long long done = 0, acc = 0;
  const Psi32 c32 = psi32_coeffs(st->psi);
  // the current distance and its psi (single precision always, FP64 when a
  // decision has needed it), recomputed only when a move is accepted
  double d_old = sqrt(ref_r2(cav[0][0], cav[0][1], cav[0][2], cav[1][0], cav[1][1], cav[1][2], len, half));
  float en32_old = cavity_psi32(c32, (float)d_old, lane);
  double en_old = 0.0;
  bool have_old = false;
  U32x4 q1{0u, 0u, 0u, 0u};
  uint32_t q2 = 0u;
  for (int k = 0; k < trials; k++) {
    // the draws of 32 trials at a time, one trial per lane
    if ((k & 31) == 0) {
      q1 = draw4(seed, (uint32_t)(k + lane), 0u, s, TAG_CAVITY);
      q2 = draw4(seed, (uint32_t)(k + lane), 1u, s, TAG_CAVITY).x;
    }
    const int src = k & 31;
    const U32x4 r1{__shfl_sync(0xffffffffu, q1.x, src), __shfl_sync(0xffffffffu, q1.y, src),
                   __shfl_sync(0xffffffffu, q1.z, src), __shfl_sync(0xffffffffu, q1.w, src)};
    const uint32_t r2x = __shfl_sync(0xffffffffu, q2, src);
    const int w = (int)(r1.x >> 31);
    // compute_dist(0, 1) before the move must lie in the allowed range
    if (d_old < cmin || d_old > cmax) {
      if (lane == 0) atomicOr(&st->status, ST_CAVITY_RANGE);
      break;
    }
    double nw[3];
    nw[0] = propose_axis(cav[w][0], centred_offset(r1.y), dr, len[0]);
    nw[1] = propose_axis(cav[w][1], centred_offset(r1.z), dr, len[1]);
    nw[2] = propose_axis(cav[w][2], centred_offset(r1.w), dr, len[2]);
    const double *c0 = w == 0 ? nw : cav[0];
    const double *c1 = w == 1 ? nw : cav[1];
    const double d_new = sqrt(ref_r2(c0[0], c0[1], c0[2], c1[0], c1[1], c1[2], len, half));
    // this lane's neighbour cell of the trial position and its count, loaded
    // now so that the load overlaps the Metropolis test
    int c = 0, nq = 0;
    float t[3] = {0.f, 0.f, 0.f};
    Slot pre0{}, pre1{};
    if (lane < 27) {
      int ci[3];
      axis_cell(__double2float_rn(nw[0]), v.sh[0], v.L32[0], v.iw[0], v.nc[0], ci[0], t[0]);
      axis_cell(__double2float_rn(nw[1]), v.sh[1], v.L32[1], v.iw[1], v.nc[1], ci[1], t[1]);
      axis_cell(__double2float_rn(nw[2]), v.sh[2], v.L32[2], v.iw[2], v.nc[2], ci[2], t[2]);
      int cx = ci[0] + ox, cy = ci[1] + oy, cz = ci[2] + oz;
      cx = cx < 0 ? cx + v.nc[0] : (cx >= v.nc[0] ? cx - v.nc[0] : cx);
      cy = cy < 0 ? cy + v.nc[1] : (cy >= v.nc[1] ? cy - v.nc[1] : cy);
      cz = cz < 0 ? cz + v.nc[2] : (cz >= v.nc[2] ? cz - v.nc[2] : cz);
      c = cx + v.nc[0] * (cy + v.nc[1] * cz);
      const int m = v.cnt[c];
      nq = m < v.cap ? m : v.cap;
      pre0 = v.slot[(size_t)c * v.cap];  // most cells hold one or two spheres: their slots
      pre1 = v.slot[(size_t)c * v.cap + 1];  // come with the count (capacity >= 16)
    }
    int decision = 1;  // the new distance leaves the allowed range
    double en_new = 0.0;
    float en32_new = 0.0f;
    bool have_new = false;
    if (d_new >= cmin && d_new <= cmax) {  // warp-uniform: every lane holds the same values
      // the reference's test u > exp(-(psi' - psi)), decided in single
      // precision unless u lies within 1e-3 (relative) of the bound
      const double u = open_unit(r2x);
      en32_new = cavity_psi32(c32, (float)d_new, lane);
      const double b32 = (double)expf(-(en32_new - en32_old));
      if (u > b32 * (1.0 + 1e-3)) {
        decision = 2;
      } else if (u < b32 * (1.0 - 1e-3)) {
        decision = 0;
      } else {
        if (!have_old) {
          en_old = cavity_psi_warp(st->psi, d_old, lane);
          have_old = true;
        }
        en_new = cavity_psi_warp(st->psi, d_new, lane);
        have_new = true;
        decision = u > exp(-(en_new - en_old)) ? 2 : 0;
      }
    }
    if (decision == 0) {
      bool ov = false;
      if (lane < 27) {
        const Slot *sl = v.slot + (size_t)c * v.cap;
        for (int q = 0; q < nq && !ov; q++) {
          const Slot o = q == 0 ? pre0 : (q == 1 ? pre1 : sl[q]);
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
      if (__any_sync(0xffffffffu, ov)) decision = 3;
    }
    if (decision == 0) {
      for (int d = 0; d < 3; d++) cav[w][d] = nw[d];
      d_old = d_new;
      en32_old = en32_new;
      en_old = en_new;
      have_old = have_new;
      if (lane == 0) {
        double *q = p.pos + 4 * (size_t)w;
        q[1] = nw[0];
        q[2] = nw[1];
        q[3] = nw[2];
      }
      acc++;
    }
    done++;
    if (trace && lane == 0) {
      const unsigned long long at = atomicAdd(&st->cav_trace_count, 1ull);
      if (at < (unsigned long long)trace_cap) {
        uint32_t *rec = trace + 8 * at;
        rec[0] = (uint32_t)s;
        rec[1] = (uint32_t)k;
        rec[2] = (uint32_t)w;
        rec[3] = r1.y;
        rec[4] = r1.z;
        rec[5] = r1.w;
        rec[6] = r2x;
        rec[7] = (uint32_t)decision;
      } else {
        atomicOr(&st->status, ST_TRACE_FULL);
      }
    }
    __syncwarp();
  }
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
