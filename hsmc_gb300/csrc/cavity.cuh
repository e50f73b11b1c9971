// The cavity umbrella potential psi(x) = ln y_GH(x) on the device, shared
// by the cavity stage (cavity.cu) and the one-block sweep (sweep_small.cu).
#pragma once

#include "engine.cuh"

namespace hsmc {

// psi(x) = lny_gh(x, pi rho / 6, 1) (src/analytic.c:34-54): the
// Grundke-Henderson cubic inside the core, ln g_VW outside, with g_VW the
// Percus-Yevick g at x / dW plus a damped oscillation (rdf_vw and rdf_py,
// src/analytic.c:79-99, 143-170), in the reference's operation order.
__device__ inline double cavity_psi(const hsmc_cavity_psi_coeffs &c, double x) {
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
__device__ inline double cavity_psi_warp(const hsmc_cavity_psi_coeffs &c, double x, int lane) {
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

__device__ inline Psi32 psi32_coeffs(const hsmc_cavity_psi_coeffs &c) {
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
__device__ inline float cavity_psi32(const Psi32 &c, float x, int lane) {
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

// The cavity trials of sweep s (cavity_part_move and cavity_check_move,
// src/moves.c:254-396) by one warp, every lane holding the same values:
//   - a cavity (one bit of the draw) is displaced as in part_move;
//   - the move is rejected when the distance between the cavities leaves
//     [cav_min, cav_max], by the Metropolis test on psi against a uniform
//     (decided in single precision unless the uniform lies within 1e-3 of
//     the bound, then in FP64), or when overlaps(nw) reports that the trial
//     position nw overlaps a particle other than the cavities;
//   - accept(w, nw) stores an accepted move.
// cav holds both cavities (updated here).  Returns false when the distance
// before a trial was outside the allowed range (the reference exits there).
// trace (8 words per trial) may be null.
template <class Overlaps, class Accept>
__device__ bool cavity_trials(const DevState *st, unsigned long long s, double (&cav)[2][3], const double *len,
                              const double *half, Overlaps &&overlaps, Accept &&accept, uint32_t *trace,
                              long long trace_cap, unsigned long long *trace_count, int *status,
                              unsigned long long &done, unsigned long long &acc) {
  const int lane = (int)(threadIdx.x & 31);
  const int trials = st->cav_trials;
  const unsigned long long seed = st->seed;
  const double dr = st->dr_max, r2lo = st->cav_r2min, r2hi = st->cav_r2max;
  const Psi32 c32 = psi32_coeffs(st->psi);
  // the current squared distance and its psi (single precision always, FP64
  // when a decision has needed it), recomputed only when a move is accepted.
  // The range tests on the distance are exact tests on r2 (cav_r2min,
  // cav_r2max), so the FP64 square root is taken only for an FP64 psi.
  double r2_old = ref_r2(cav[0][0], cav[0][1], cav[0][2], cav[1][0], cav[1][1], cav[1][2], len, half);
  float en32_old = cavity_psi32(c32, sqrtf(__double2float_rn(r2_old)), lane);
  double en_old = 0.0;
  bool have_old = false;
  U32x4 q1{0u, 0u, 0u, 0u};
  uint32_t q2 = 0u;
  for (int k = 0; k < trials; k++) {
    if ((k & 31) == 0) {  // the draws of 32 trials at a time, one trial per lane
      q1 = draw4(seed, (uint32_t)(k + lane), 0u, s, TAG_CAVITY);
      q2 = draw4(seed, (uint32_t)(k + lane), 1u, s, TAG_CAVITY).x;
    }
    const int src = k & 31;
    const U32x4 r1{__shfl_sync(0xffffffffu, q1.x, src), __shfl_sync(0xffffffffu, q1.y, src),
                   __shfl_sync(0xffffffffu, q1.z, src), __shfl_sync(0xffffffffu, q1.w, src)};
    const uint32_t r2x = __shfl_sync(0xffffffffu, q2, src);
    const int w = (int)(r1.x >> 31);
    // compute_dist(0, 1) before the move must lie in the allowed range
    if (r2_old < r2lo || r2_old > r2hi) {
      if (lane == 0) atomicOr(status, ST_CAVITY_RANGE);
      return false;
    }
    double nw[3];
    nw[0] = propose_axis(cav[w][0], centred_offset(r1.y), dr, len[0]);
    nw[1] = propose_axis(cav[w][1], centred_offset(r1.z), dr, len[1]);
    nw[2] = propose_axis(cav[w][2], centred_offset(r1.w), dr, len[2]);
    const double *c0 = w == 0 ? nw : cav[0];
    const double *c1 = w == 1 ? nw : cav[1];
    const double r2_new = ref_r2(c0[0], c0[1], c0[2], c1[0], c1[1], c1[2], len, half);
    int decision = 1;  // the new distance leaves the allowed range
    double en_new = 0.0;
    float en32_new = 0.0f;
    bool have_new = false;
    if (r2_new >= r2lo && r2_new <= r2hi) {
      // the reference's test u > exp(-(psi' - psi))
      const double u = open_unit(r2x);
      en32_new = cavity_psi32(c32, sqrtf(__double2float_rn(r2_new)), lane);
      const double b32 = (double)expf(-(en32_new - en32_old));
      if (u > b32 * (1.0 + 1e-3)) {
        decision = 2;
      } else if (u < b32 * (1.0 - 1e-3)) {
        decision = 0;
      } else {
        if (!have_old) {
          en_old = cavity_psi_warp(st->psi, sqrt(r2_old), lane);
          have_old = true;
        }
        en_new = cavity_psi_warp(st->psi, sqrt(r2_new), lane);
        have_new = true;
        decision = u > exp(-(en_new - en_old)) ? 2 : 0;
      }
    }
    if (decision == 0 && overlaps(nw)) decision = 3;
    if (decision == 0) {
      for (int d = 0; d < 3; d++) cav[w][d] = nw[d];
      r2_old = r2_new;
      en32_old = en32_new;
      en_old = en_new;
      have_old = have_new;
      accept(w, nw);
      acc++;
    }
    done++;
    if (trace && lane == 0) {
      const unsigned long long at = atomicAdd(trace_count, 1ull);
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
        atomicOr(status, ST_TRACE_FULL);
      }
    }
    __syncwarp();
  }
  return true;
}

}  // namespace hsmc
