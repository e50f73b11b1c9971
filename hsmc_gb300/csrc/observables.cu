// Observables sampled between sweeps, all computed on the current cell
// layout of the sweep grid with a stencil wide enough for their cutoff:
//   k_pair_hist     g(r) and the virial contact histogram: integer pair
//                   counts, warp-aggregated into shared-memory bins
//                   (rdf_hist_compute src/compute_rdf.c:110-128,
//                   pressv_compute_hist src/compute_press.c:123-165)
//   k_scaled_scan   overlap of the configuration scaled by sf < 1, for the
//                   thermodynamic pressure and the NpT volume move
//                   (presst_compute_hist src/compute_press.c:243-273,
//                   vol_move src/moves.c:104-112)
//   k_widom         test-particle insertions (src/compute_widom_chem_pot.c:44-120)
//   k_replay        check_overlap on given trial positions, screened as the move
//                   pass screens a trial (src/moves.c:157-212)
//   k_ql            Steinhardt q_l per particle (src/compute_order_parameter.c:99-229)
// Every decision that the reference takes in FP64 is taken here either in
// FP64 with its operation order, or in single precision where the single
// precision value lies farther from the decision's threshold than its error
// bound (the guard band), so that both give the same answer.
#include <cooperative_groups.h>

#include "cellview.cuh"
#include "df64.cuh"
#include "screen.cuh"

namespace cg = cooperative_groups;

namespace hsmc {

// ------------------------------------------------------------ pair counts
constexpr int HIST_SMEM_BINS = 4096;

// In a batch (BATCH), blockIdx.y is the replica: its pointers come from reps,
// its counts go to counts + replica * nbins, and its stencil follows its grid.
template <bool BATCH>
__global__ void __launch_bounds__(256) k_pair_hist(SysPtrs p1, const SysPtrs *reps, Stencil s1, double bin,
                                                   double rmax, int nbins, unsigned long long *counts1, float cut2) {
  const SysPtrs p = BATCH ? reps[blockIdx.y] : p1;
  unsigned long long *counts = BATCH ? counts1 + (size_t)blockIdx.y * nbins : counts1;
  Stencil s = s1;
  if (BATCH) {
    for (int d = 0; d < 3; d++) {
      const int nc = p.box->nc[d];
      int kk = (int)ceil((rmax + 1e-3) * nc / p.box->len[d]);
      kk = kk < 1 ? 1 : kk;
      s.k[d] = (2 * kk + 1 >= nc) ? -1 : kk;
    }
  }
  __shared__ unsigned int sh[HIST_SMEM_BINS];
  const bool use_sh = nbins <= HIST_SMEM_BINS;
  if (use_sh)
    for (int b = threadIdx.x; b < nbins; b += blockDim.x) sh[b] = 0;
  __syncthreads();
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool bad = false;
  if (i < p.n) {
    double x, y, z;
    load_xyz(p.pos, i, x, y, z);
    float x32, y32, z32;  // grid coordinates, as the slots hold them
    grid_coords(v, x, y, z, x32, y32, z32);
    for_each_near(v, s, x, y, z, cut2, [&](const Slot &o) {
      if (o.id == i) return false;
      if (approx_r2(x32, y32, z32, o, v.L32) > cut2) return false;
      double ox, oy, oz;
      load_xyz(p.pos, o.id, ox, oy, oz);
      const double r = __dsqrt_rn(ref_r2(x, y, z, ox, oy, oz, len, half));
      if (r < rmax) {
        const int b = (int)__ddiv_rn(__dsub_rn(r, 1.0), bin);
        if (b < 0 || b >= nbins) {
          bad = true;
          return false;
        }
        if (use_sh) {
          // warp aggregation: one shared-memory atomic per distinct bin
          cg::coalesced_group active = cg::coalesced_threads();
          cg::coalesced_group same = cg::labeled_partition(active, b);
          if (same.thread_rank() == 0) atomicAdd(&sh[b], same.size());
        } else {
          atomicAdd(counts + b, 1ull);
        }
      }
      return false;
    });
  }
  if (bad) atomicOr(&p.st->status, ST_BAD_BIN);
  __syncthreads();
  if (use_sh)
    for (int b = threadIdx.x; b < nbins; b += blockDim.x)
      if (sh[b]) atomicAdd(counts + b, (unsigned long long)sh[b]);
}

// The same counts with the reference's bin formula evaluated only where it
// is needed.  thr[k] (k = 1..nbins) is the smallest double r2 whose bin
// (int)((sqrt(r2) - 1) / dr) reaches k, thr[nbins + 1] the smallest whose
// root reaches rmax (thr[0] = 1), found on the host with the same correctly
// rounded operations (pair_thresholds, api.cu), so that for every double
// r2 in [1, thr[nbins]) the bin is the number of thresholds at or below it.
// A pair's single-precision r2 (grid coordinates, the cell's periodic
// image) is within band (1 + r2) of the reference's FP64 r2 (the move
// pass's guard band, scaled for distances up to rmax), so a pair whose
// single-precision r2 is farther than that from every threshold is binned
// without FP64 work; the others take the reference's FP64 distance.  Each
// unordered pair is visited once (half stencil; in the own cell j > i) and
// counts 2, as the reference's +2.0 per pair: the FP64 distance of (i, j)
// and (j, i) is the same number.  Needs a stencil narrower than the grid.
constexpr int FAST_BINS = 2048;

__device__ __forceinline__ int exact_bin(double r2, const double *thr, int nbins, double bin, double rmax, int guess,
                                         bool &bad) {
  if (r2 < 1.0 || !(r2 < thr[nbins])) {  // overlapping or beyond the last bin: the reference's formula
    const double r = __dsqrt_rn(r2);
    if (!(r < rmax)) return -1;
    const int b = (int)__ddiv_rn(__dsub_rn(r, 1.0), bin);
    if (b < 0 || b >= nbins) {
      bad = true;
      return -1;
    }
    return b;
  }
  // thr[0] = 1 <= r2 < thr[nbins]: the largest k with thr[k] <= r2 (positive
  // doubles order as their bit patterns)
  const long long x = __double_as_longlong(r2);
  int k = guess < 0 ? 0 : (guess >= nbins ? nbins - 1 : guess);
  while (k > 0 && __double_as_longlong(__ldg(thr + k)) > x) k--;
  while (k + 1 < nbins && __double_as_longlong(__ldg(thr + k + 1)) <= x) k++;
  return k;
}

// A pair that single precision cannot bin waits in its warp's queue, and
// the warp bins 32 of them at a time with every lane on the FP64 path: left
// in the pair loop, the FP64 instructions of one or two lanes would stall
// the warp in most iterations (about one pair in twelve is near a threshold
// at r_max = 5).  The pair loop runs to the warp's fullest cell, so the
// lanes are converged at each queue step.
constexpr int PAIR_QUEUE = 64;  // per warp: up to 31 waiting + 32 appended

__device__ __forceinline__ void bin_pending(const SysPtrs &p, const int4 e, const double len[3],
                                            const double half[3], const double *thr, int nbins, double bin,
                                            double rmax, unsigned int *sh, bool &bad) {
  double x, y, z, ox, oy, oz;
  load_xyz(p.pos, e.x, x, y, z);
  load_xyz(p.pos, e.y, ox, oy, oz);
  const int bn = exact_bin(ref_r2(x, y, z, ox, oy, oz, len, half), thr, nbins, bin, rmax, e.z, bad);
  if (bn >= 0) atomicAdd(&sh[bn], 2u);
}

__global__ void __launch_bounds__(256) k_pair_hist_fast(SysPtrs p, Stencil s, double bin, double rmax, int nbins,
                                                        unsigned long long *counts, float cut2, const double *thr) {
  __shared__ unsigned int sh[FAST_BINS];
  __shared__ float thr_f[FAST_BINS + 2];
  __shared__ int4 queue[256 / 32][PAIR_QUEUE];
  for (int b = threadIdx.x; b < nbins; b += blockDim.x) sh[b] = 0;
  for (int k = threadIdx.x; k < nbins + 2; k += blockDim.x) thr_f[k] = (float)__ldg(thr + k);
  __syncthreads();
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const float band = bx->band;
  const float inv_bin = (float)(1.0 / bin);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int4 *q = queue[threadIdx.x >> 5];
  int qn = 0;  // the warp's waiting pairs, the same in every lane
  bool bad = false;
  const bool live = i < p.n;
  int ci[3] = {0, 0, 0};
  float t[3] = {0.f, 0.f, 0.f};
  StencilGap gap;
  if (live) {
    double x, y, z;
    load_xyz(p.pos, i, x, y, z);
    axis_cell(__double2float_rn(x), v.sh[0], v.L32[0], v.iw[0], v.nc[0], ci[0], t[0]);
    axis_cell(__double2float_rn(y), v.sh[1], v.L32[1], v.iw[1], v.nc[1], ci[1], t[1]);
    axis_cell(__double2float_rn(z), v.sh[2], v.L32[2], v.iw[2], v.nc[2], ci[2], t[2]);
    gap.init(ci, t, v.w);
  }
  for (int a = 0; a <= s.k[2]; a++) {
    int cz = ci[2] + a;
    const float imz = cz >= v.nc[2] ? v.L32[2] : 0.f;
    cz -= cz >= v.nc[2] ? v.nc[2] : 0;
    const float gz = gap.sq(2, a);
    if (__all_sync(0xffffffffu, !live || gz > cut2)) break;  // farther a only farther
    for (int b = (a == 0 ? 0 : -s.k[1]); b <= s.k[1]; b++) {
      int cy = ci[1] + b;
      const float imy = cy < 0 ? -v.L32[1] : (cy >= v.nc[1] ? v.L32[1] : 0.f);
      cy += cy < 0 ? v.nc[1] : (cy >= v.nc[1] ? -v.nc[1] : 0);
      const float gzy = gz + gap.sq(1, b);
      if (__all_sync(0xffffffffu, !live || gzy > cut2)) continue;
      for (int e = ((a == 0 && b == 0) ? 0 : -s.k[0]); e <= s.k[0]; e++) {
        int cx = ci[0] + e;
        const float imx = cx < 0 ? -v.L32[0] : (cx >= v.nc[0] ? v.L32[0] : 0.f);
        cx += cx < 0 ? v.nc[0] : (cx >= v.nc[0] ? -v.nc[0] : 0);
        const bool own = a == 0 && b == 0 && e == 0;
        const int c = cx + v.nc[0] * (cy + v.nc[1] * cz);
        int n = 0;
        if (live && gzy + gap.sq(0, e) <= cut2) {  // the cell's nearest point is within the cut
          const int m = v.cnt[c];
          n = m < v.cap ? m : v.cap;  // an overfull cell was flagged by the build
        }
        const Slot *sl = v.slot + (size_t)c * v.cap;
        const int n_warp = __reduce_max_sync(0xffffffffu, n);
        for (int k0 = 0; k0 < n_warp; k0++) {
          int bn = -1, guess = 0, j = 0;
          bool wait = false;
          if (k0 < n) {
            const Slot o = sl[k0];
            const float4 ent = imaged_entry(o, imx, imy, imz);
            const float r2f = dist2(t[0], t[1], t[2], ent);
            if (!(own && o.id <= i) && r2f <= cut2) {
              // single precision where it decides: the bin whose thresholds
              // lie farther than the error bound on both sides.  The bin is
              // estimated from sqrt(r2) and only checked against its two
              // thresholds: an estimate off by one lies within the error
              // bound of a threshold, and such a pair is queued anyway
              const float err = band * (1.0f + r2f) + 2.4e-7f * (1.0f + r2f);
              int k = (int)((sqrtf(r2f) - 1.0f) * inv_bin);
              k = k < 0 ? 0 : (k > nbins - 1 ? nbins - 1 : k);
              if (r2f - err > thr_f[nbins + 1]) {
                // beyond rmax
              } else if (r2f - err > thr_f[k] && r2f + err < thr_f[k + 1] && k + 1 <= nbins) {
                bn = k;
              } else {
                wait = true;
                guess = k;
                j = o.id;
              }
            }
          }
          if (bn >= 0) atomicAdd(&sh[bn], 2u);
          const unsigned wq = __ballot_sync(0xffffffffu, wait);
          if (wait) q[qn + __popc(wq & ((1u << lane) - 1u))] = make_int4(i, j, guess, 0);
          qn += __popc(wq);
          if (qn >= 32) {
            __syncwarp();
            qn -= 32;
            const int4 w = q[qn + lane];
            __syncwarp();
            bin_pending(p, w, len, half, thr, nbins, bin, rmax, sh, bad);
          }
        }
      }
    }
  }
  __syncwarp();
  if (lane < qn) bin_pending(p, q[lane], len, half, thr, nbins, bin, rmax, sh, bad);
  if (bad) atomicOr(&p.st->status, ST_BAD_BIN);
  __syncthreads();
  for (int b = threadIdx.x; b < nbins; b += blockDim.x)
    if (sh[b]) atomicAdd(counts + b, (unsigned long long)sh[b]);
}

// thr: the r2 thresholds of the bins (nbins + 2 doubles, see above) or
// nullptr for the exact per-pair FP64 kernel, which also serves more bins
// than FAST_BINS and grids too small for a half stencil.
void launch_pair_hist(const SysPtrs &p, double bin, double rmax, int nbins, unsigned long long *counts,
                      int stencil[3], cudaStream_t st, const double *thr) {
  Stencil s{{stencil[0], stencil[1], stencil[2]}};
  const float cut = (float)rmax + 1e-3f;
  const int blocks = (p.n + 255) / 256;
  const bool fast = thr && nbins <= FAST_BINS && stencil[0] >= 0 && stencil[1] >= 0 && stencil[2] >= 0;
  if (fast)
    k_pair_hist_fast<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(p, s, bin, rmax, nbins, counts, cut * cut, thr);
  else
    k_pair_hist<false><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(p, nullptr, s, bin, rmax, nbins, counts, cut * cut);
}

void launch_pair_hist_batch(const SysPtrs *reps, int n_reps, int max_n, double bin, double rmax, int nbins,
                            unsigned long long *counts, cudaStream_t st) {
  const float cut = (float)rmax + 1e-3f;
  const dim3 grid((unsigned)((max_n + 255) / 256), (unsigned)n_reps);
  k_pair_hist<true><<<grid, 256, 0, st>>>(SysPtrs{}, reps, Stencil{{0, 0, 0}}, bin, rmax, nbins, counts, cut * cut);
}

// ------------------------------------------------------- scaled overlap
constexpr int MAX_SF = 256;
__constant__ double c_sf[MAX_SF];
__constant__ float c_sf2f[MAX_SF];  // (float)(sf * sf)

__global__ void __launch_bounds__(256) k_scaled_scan(SysPtrs p, Stencil s, int n_sf, float cut2) {
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long m[4] = {0ull, 0ull, 0ull, 0ull};
  if (i < p.n) {
    double x, y, z;
    load_xyz(p.pos, i, x, y, z);
    float x32, y32, z32;  // grid coordinates, as the slots hold them
    grid_coords(v, x, y, z, x32, y32, z32);
    // the scaled single-precision r^2 decides outside twice the guard band of
    // contact (scaling by sf <= 1 shrinks the screen's error); inside it the
    // reference's scaled FP64 distance does
    const float lo = 1.0f - 2.0f * v.band, hi = 1.0f + 2.0f * v.band;
    for_each_near<false>(v, s, x, y, z, cut2, [&](const Slot &o) {
      if (o.id == i) return false;
      const float r2f = approx_r2(x32, y32, z32, o, v.L32);
      if (r2f > cut2) return false;
      bool loaded = false;
      double ox = 0.0, oy = 0.0, oz = 0.0;
      for (int k = 0; k < n_sf; k++) {
        const unsigned long long bit = 1ull << (k & 63);
        if (m[k >> 6] & bit) continue;
        const float est = r2f * c_sf2f[k];
        if (est < lo) {
          m[k >> 6] |= bit;
          continue;
        }
        if (est > hi) continue;
        if (!loaded) {
          load_xyz(p.pos, o.id, ox, oy, oz);
          loaded = true;
        }
        if (ref_r2_scaled(x, y, z, ox, oy, oz, len, c_sf[k]) < 1.0) m[k >> 6] |= bit;
      }
      return false;
    });
  }
  for (int w = 0; w < 4; w++) {
    unsigned long long r = m[w];
    for (int o = 16; o > 0; o >>= 1) r |= __shfl_xor_sync(0xffffffffu, r, o);
    if ((threadIdx.x & 31) == 0 && r) atomicOr(&p.st->scan_mask[w], r);
  }
}

// The same scan over a half stencil (each unordered pair once: the scaled
// FP64 distance of (i, j) and (j, i) is the same number), warp by warp in
// step as the pair counts go, with the pairs inside the band of a scaled
// contact queued per warp and decided 32 at a time in FP64.  The result is
// an OR over pairs, so a warp stops once every scale factor has an overlap
// somewhere: after each stencil cell it publishes the bits it found and
// reads those of the whole grid.  Needs a stencil narrower than the grid.
__device__ __forceinline__ void scaled_pending(const SysPtrs &p, const int4 e, const double len[3], int n_sf,
                                               float lo, float hi, unsigned long long m[4]) {
  double x, y, z, ox, oy, oz;
  load_xyz(p.pos, e.x, x, y, z);
  load_xyz(p.pos, e.y, ox, oy, oz);
  const float r2f = __int_as_float(e.z);
  for (int k = 0; k < n_sf; k++) {
    const unsigned long long bit = 1ull << (k & 63);
    if (m[k >> 6] & bit) continue;
    const float est = r2f * c_sf2f[k];
    if (est < lo || est > hi) continue;  // decided in single precision at the queueing
    if (ref_r2_scaled(x, y, z, ox, oy, oz, len, c_sf[k]) < 1.0) m[k >> 6] |= bit;
  }
}

__global__ void __launch_bounds__(256) k_scaled_scan_fast(SysPtrs p, Stencil s, int n_sf, float cut2) {
  __shared__ int4 queue[256 / 32][PAIR_QUEUE];
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int4 *q = queue[threadIdx.x >> 5];
  int qn = 0;
  const bool live = i < p.n;
  // the scaled single-precision r^2 decides outside twice the guard band of
  // contact (scaling by sf <= 1 shrinks the screen's error)
  const float lo = 1.0f - 2.0f * v.band, hi = 1.0f + 2.0f * v.band;
  unsigned long long m[4] = {0ull, 0ull, 0ull, 0ull}, full[4];
#pragma unroll
  for (int w = 0; w < 4; w++) {
    const int b = n_sf - 64 * w;  // bits of word w in use
    full[w] = b >= 64 ? ~0ull : (b > 0 ? (1ull << b) - 1ull : 0ull);
  }
  const int nw = (n_sf + 63) >> 6;
  unsigned long long *gmask = p.st->scan_mask;
  int ci[3] = {0, 0, 0};
  float t[3] = {0.f, 0.f, 0.f};
  StencilGap gap;
  if (live) {
    double x, y, z;
    load_xyz(p.pos, i, x, y, z);
    axis_cell(__double2float_rn(x), v.sh[0], v.L32[0], v.iw[0], v.nc[0], ci[0], t[0]);
    axis_cell(__double2float_rn(y), v.sh[1], v.L32[1], v.iw[1], v.nc[1], ci[1], t[1]);
    axis_cell(__double2float_rn(z), v.sh[2], v.L32[2], v.iw[2], v.nc[2], ci[2], t[2]);
    gap.init(ci, t, v.w);
  }
  bool done = false;
  for (int a = 0; a <= s.k[2] && !done; a++) {
    int cz = ci[2] + a;
    const float imz = cz >= v.nc[2] ? v.L32[2] : 0.f;
    cz -= cz >= v.nc[2] ? v.nc[2] : 0;
    const float gz = gap.sq(2, a);
    if (__all_sync(0xffffffffu, !live || gz > cut2)) break;
    for (int b = (a == 0 ? 0 : -s.k[1]); b <= s.k[1] && !done; b++) {
      int cy = ci[1] + b;
      const float imy = cy < 0 ? -v.L32[1] : (cy >= v.nc[1] ? v.L32[1] : 0.f);
      cy += cy < 0 ? v.nc[1] : (cy >= v.nc[1] ? -v.nc[1] : 0);
      const float gzy = gz + gap.sq(1, b);
      if (__all_sync(0xffffffffu, !live || gzy > cut2)) continue;
      for (int e = ((a == 0 && b == 0) ? 0 : -s.k[0]); e <= s.k[0] && !done; e++) {
        int cx = ci[0] + e;
        const float imx = cx < 0 ? -v.L32[0] : (cx >= v.nc[0] ? v.L32[0] : 0.f);
        cx += cx < 0 ? v.nc[0] : (cx >= v.nc[0] ? -v.nc[0] : 0);
        const bool own = a == 0 && b == 0 && e == 0;
        const int c = cx + v.nc[0] * (cy + v.nc[1] * cz);
        int n = 0;
        if (live && gzy + gap.sq(0, e) <= cut2) {
          const int mm = v.cnt[c];
          n = mm < v.cap ? mm : v.cap;
        }
        const Slot *sl = v.slot + (size_t)c * v.cap;
        const int n_warp = __reduce_max_sync(0xffffffffu, n);
        for (int k0 = 0; k0 < n_warp; k0++) {
          bool wait = false;
          int j = 0;
          float r2q = 0.f;
          if (k0 < n) {
            const Slot o = sl[k0];
            const float4 ent = imaged_entry(o, imx, imy, imz);
            const float r2f = dist2(t[0], t[1], t[2], ent);
            if (!(own && o.id <= i) && r2f <= cut2) {
              for (int k = 0; k < n_sf; k++) {
                const unsigned long long bit = 1ull << (k & 63);
                if (m[k >> 6] & bit) continue;
                const float est = r2f * c_sf2f[k];
                if (est < lo) m[k >> 6] |= bit;
                else if (est <= hi) wait = true;
              }
              j = o.id;
              r2q = r2f;
            }
          }
          const unsigned wq = __ballot_sync(0xffffffffu, wait);
          if (wait) q[qn + __popc(wq & ((1u << lane) - 1u))] = make_int4(i, j, __float_as_int(r2q), 0);
          qn += __popc(wq);
          if (qn >= 32) {
            __syncwarp();
            qn -= 32;
            const int4 w = q[qn + lane];
            __syncwarp();
            scaled_pending(p, w, len, n_sf, lo, hi, m);
          }
        }
        // publish this warp's bits; stop once the grid has all of them
        bool all = true;
#pragma unroll
        for (int w = 0; w < 4; w++) {
          if (w >= nw) break;
          unsigned long long r = m[w];
          for (int o = 16; o > 0; o >>= 1) r |= __shfl_xor_sync(0xffffffffu, r, o);
          unsigned long long g = 0ull;
          if (lane == 0) {
            const unsigned long long seen = *(volatile unsigned long long *)(gmask + w);
            g = (r & ~seen) ? atomicOr(gmask + w, r) | r : seen;
          }
          g = __shfl_sync(0xffffffffu, g, 0);
          all = all && ((g & full[w]) == full[w]);
        }
        done = all;
      }
    }
  }
  __syncwarp();
  if (lane < qn) scaled_pending(p, q[lane], len, n_sf, lo, hi, m);
  for (int w = 0; w < 4; w++) {
    unsigned long long r = m[w];
    for (int o = 16; o > 0; o >>= 1) r |= __shfl_xor_sync(0xffffffffu, r, o);
    if (lane == 0 && r) atomicOr(gmask + w, r);
  }
}

void launch_scaled_scan(const SysPtrs &p, const double *sf, int n_sf, int stencil[3], cudaStream_t st) {
  double smallest = 1.0;
  for (int k = 0; k < n_sf; k++) smallest = sf[k] < smallest ? sf[k] : smallest;
  cudaMemcpyToSymbolAsync(c_sf, sf, sizeof(double) * (size_t)n_sf, 0, cudaMemcpyHostToDevice, st);
  float sf2f[MAX_SF];
  for (int k = 0; k < n_sf; k++) sf2f[k] = (float)(sf[k] * sf[k]);
  cudaMemcpyToSymbolAsync(c_sf2f, sf2f, sizeof(float) * (size_t)n_sf, 0, cudaMemcpyHostToDevice, st);
  Stencil s{{stencil[0], stencil[1], stencil[2]}};
  const float cut = (float)(1.0 / smallest) + 1e-3f;
  const int blocks = (p.n + 255) / 256;
  if (stencil[0] >= 0 && stencil[1] >= 0 && stencil[2] >= 0)
    k_scaled_scan_fast<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(p, s, n_sf, cut * cut);
  else
    k_scaled_scan<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(p, s, n_sf, cut * cut);
}

// ----------------------------------------------------------------- Widom
__global__ void __launch_bounds__(256, 3) k_widom(SysPtrs p, long long n, unsigned long long seq, const double *pos_in,
                                               uint8_t *ov_out) {
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const Stencil s{{1, 1, 1}};
  const unsigned long long seed = p.st->seed;
  unsigned long long ok = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    double x, y, z;
    if (pos_in) {
      x = pos_in[3 * k];
      y = pos_in[3 * k + 1];
      z = pos_in[3 * k + 2];
    } else {
      const U32x4 r = draw4(seed, (uint32_t)k, (uint32_t)(k >> 32), seq, TAG_WIDOM);
      x = __dmul_rn(open_unit(r.x), len[0]);
      y = __dmul_rn(open_unit(r.y), len[1]);
      z = __dmul_rn(open_unit(r.z), len[2]);
    }
    const bool ov = point_overlaps(v, p, s, x, y, z, -1, len, half);
    if (ov_out) ov_out[k] = ov ? 1 : 0;
    ok += ov ? 0 : 1;
  }
  ok = warp_sum_u64(ok);
  if ((threadIdx.x & 31) == 0 && ok) atomicAdd(&p.st->widom_ok, ok);
}

void launch_widom(const SysPtrs &p, long long n, unsigned long long seq, const double *pos_in, uint8_t *ov_out,
                  cudaStream_t st) {
  long long blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  k_widom<<<(int)blocks, 256, 0, st>>>(p, n, seq, pos_in, ov_out);
}

// ----------------------------------------------------------------- replay
// check_overlap (src/moves.c:157-212) at given trial positions, screened
// exactly as a move-pass trial is: the position's grid coordinates against
// the slots of its cell and of the 26 cells around it (imaged across the
// periodic faces), single precision outside the guard band of contact, the
// reference's FP64 distance inside it (screen.cuh).  A replayed decision
// therefore tests the band the move pass relies on, at any box size.
__global__ void __launch_bounds__(256) k_replay(SysPtrs p, const int *ids, const double *pos_in, int n,
                                                uint8_t *ov_out) {
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const float lo = 1.0f - bx->band, hi = 1.0f + bx->band;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const double x = pos_in[3 * k], y = pos_in[3 * k + 1], z = pos_in[3 * k + 2];
  const int skip = ids[k];
  int ix, iy, iz;
  float ux, uy, uz;
  axis_cell(__double2float_rn(x), v.sh[0], v.L32[0], v.iw[0], v.nc[0], ix, ux);
  axis_cell(__double2float_rn(y), v.sh[1], v.L32[1], v.iw[1], v.nc[1], iy, uy);
  axis_cell(__double2float_rn(z), v.sh[2], v.L32[2], v.iw[2], v.nc[2], iz, uz);
  const int c = ix + v.nc[0] * (iy + v.nc[1] * iz);
  bool ov = false;
  auto screen = [&](const float4 &q) {
    if (ov || __float_as_int(q.w) == skip) return;
    const float r2 = dist2(ux, uy, uz, q);
    if (r2 < lo) {
      ov = true;
    } else if (r2 <= hi) {
      double ox, oy, oz;
      load_xyz(p.pos, __float_as_int(q.w), ox, oy, oz);
      ov = ref_r2(x, y, z, ox, oy, oz, len, half) < 1.0;
    }
  };
  {
    const int m = v.cnt[c];
    const int nn = m < v.cap ? m : v.cap;
    for (int q = 0; q < nn; q++) {
      const Slot o = v.slot[(size_t)c * v.cap + q];
      screen(make_float4(o.x, o.y, o.z, __int_as_float(o.id)));
    }
  }
  for (int o26 = 0; o26 < 26 && !ov; o26++) {
    const unsigned code = c_nbr[o26];
    const int nb = neighbour_cell(code, ix, iy, iz, c, v.nc, false);
    float imx, imy, imz;
    image_of(code, ix, iy, iz, v.nc, v.L32, imx, imy, imz);
    const int m = v.cnt[nb];
    const int nn = m < v.cap ? m : v.cap;
    for (int q = 0; q < nn; q++) screen(imaged_entry(v.slot[(size_t)nb * v.cap + q], imx, imy, imz));
  }
  ov_out[k] = ov ? 1 : 0;
}

void launch_overlap_replay(const SysPtrs &p, const int *ids, const double *pos_in, int n, uint8_t *ov_out,
                           cudaStream_t st) {
  const int blocks = (n + 255) / 256;
  k_replay<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(p, ids, pos_in, n, ov_out);
}

// -------------------------------------------------------------------- q_l
// Normalised associated Legendre functions by the standard recurrences
// (Pbar_m^m from Pbar_{m-1}^{m-1}, Pbar_{m+1}^m, then the three-term
// recurrence in l), with the coefficients tabulated on the host per call,
// as doubles and as double-float pairs (df64.cuh).
constexpr int QL_LMAX = 12;
struct QlCoef {
  F2 neg_diag[QL_LMAX + 1];            // -sqrt((2m+1)/(2m)), m >= 1
  F2 first[QL_LMAX + 1];               // sqrt(2m+3)
  F2 a[QL_LMAX + 1][QL_LMAX + 1];      // a[l][m]
  F2 b[QL_LMAX + 1][QL_LMAX + 1];      // b[l][m]
};
__constant__ QlCoef c_ql;

// One bond's contribution to q_lm, m = 0..l (Y_lm by the recurrences of
// QlCoef; cos m phi, sin m phi by the angle-addition recurrence).  The
// angles' cosines and sines come from FP64 (two reciprocals and a square
// root); the recurrences and the sums run in double-float arithmetic on the
// FP32 pipe (about 48 bits: q_l within about 1e-14 of the FP64 recurrences),
// which bounded this kernel in FP64.
// LT > 0: l = LT at compile time (the loops unroll and the sums stay in
// registers); LT = 0: l from the argument.
template <int LT>
__device__ __forceinline__ void ql_bond(double dx, double dy, double dz, double r, int l_arg, F2 *re, F2 *im) {
  const int l = LT > 0 ? LT : l_arg;
  const double inv_r = 1.0 / r;
  const double rho = sqrt(dx * dx + dy * dy);
  const double inv_rho = rho > 0.0 ? 1.0 / rho : 0.0;
  const F2 ct = f2_of(dz * inv_r), st = f2_of(rho * inv_r);
  const F2 cp = f2_of(rho > 0.0 ? dx * inv_rho : 1.0), sp = f2_of(rho > 0.0 ? dy * inv_rho : 0.0);
  F2 pmm = f2_of(0.28209479177387814), cm = F2{1.0f, 0.0f}, sm = F2{0.0f, 0.0f};  // 1 / sqrt(4 pi)
#pragma unroll
  for (int m = 0; m <= (LT > 0 ? LT : QL_LMAX); m++) {
    if (LT == 0 && m > l) break;
    if (m > 0) {
      pmm = f2_mul(f2_mul(pmm, c_ql.neg_diag[m]), st);
      const F2 c2 = f2_sub(f2_mul(cm, cp), f2_mul(sm, sp));
      sm = f2_add(f2_mul(sm, cp), f2_mul(cm, sp));
      cm = c2;
    }
    F2 plm = pmm;
    if (l > m) {
      F2 p2 = pmm, p1 = f2_mul(f2_mul(ct, c_ql.first[m]), pmm);
#pragma unroll
      for (int ll = m + 2; ll <= (LT > 0 ? LT : QL_LMAX); ll++) {
        if (LT == 0 && ll > l) break;
        const F2 pn = f2_mul(c_ql.a[ll][m], f2_sub(f2_mul(ct, p1), f2_mul(c_ql.b[ll][m], p2)));
        p2 = p1;
        p1 = pn;
      }
      plm = p1;
    }
    re[m] = f2_add(re[m], f2_mul(plm, cm));
    im[m] = f2_add(im[m], f2_mul(plm, sm));
  }
}

// Per particle: first its bonds (neighbours with r <= rc: the
// single-precision r^2 decides outside a guard band of rc^2, the
// reference's FP64 distance inside it), kept as ids in shared memory; then
// the FP64 harmonics of one bond per lane per step.  A warp's FP64 sequence
// then runs once per bond of its busiest lane, not once per candidate
// neighbour of any lane.  Bonds are summed in the order found (the first
// QL_MAXB; a particle with more adds the rest as it finds them).
constexpr int QL_MAXB = 64;

// Five blocks an SM for l compiled in (96 registers, no spills): the
// double-float chains are latency-bound, and more warps hide more of it.
template <int LT>
__global__ void __launch_bounds__(128, LT > 0 ? 5 : 1) k_ql(SysPtrs p, Stencil s, int l_arg, double rc, float cut2,
                                                             double *q_out) {
  const int l = LT > 0 ? LT : l_arg;
  __shared__ int bond_id[QL_MAXB][128];
  const CellView v = current_view(p);
  const Box *bx = p.box;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  double x, y, z;
  load_xyz(p.pos, i, x, y, z);
  float x32, y32, z32;  // grid coordinates, as the slots hold them
  grid_coords(v, x, y, z, x32, y32, z32);
  constexpr int NM = LT > 0 ? LT + 1 : QL_LMAX + 1;
  F2 re[NM], im[NM];
#pragma unroll
  for (int m = 0; m < NM; m++) re[m] = im[m] = F2{0.0f, 0.0f};
  int bonds = 0;
  const float rc2f = (float)(rc * rc);
  const float err = v.band * (1.0f + rc2f) + 2.4e-7f * (1.0f + rc2f);
  for_each_near(v, s, x, y, z, cut2, [&](const Slot &o) {
    if (o.id == i) return false;
    const float r2f = approx_r2(x32, y32, z32, o, v.L32);
    if (r2f > cut2 || r2f > rc2f + err) return false;
    if (r2f >= rc2f - err || bonds >= QL_MAXB) {
      double ox, oy, oz;
      load_xyz(p.pos, o.id, ox, oy, oz);
      const double dx = min_image(__dsub_rn(x, ox), len[0], half[0]);
      const double dy = min_image(__dsub_rn(y, oy), len[1], half[1]);
      const double dz = min_image(__dsub_rn(z, oz), len[2], half[2]);
      const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
      if (!(r <= rc)) return false;
      if (bonds >= QL_MAXB) {  // beyond the list: summed now
        ql_bond<LT>(dx, dy, dz, r, l, re, im);
        bonds++;
        return false;
      }
    }
    bond_id[bonds][threadIdx.x] = o.id;
    bonds++;
    return false;
  });
  const int listed = bonds < QL_MAXB ? bonds : QL_MAXB;
  for (int b = 0; b < listed; b++) {
    double ox, oy, oz;
    load_xyz(p.pos, bond_id[b][threadIdx.x], ox, oy, oz);
    const double dx = min_image(__dsub_rn(x, ox), len[0], half[0]);
    const double dy = min_image(__dsub_rn(y, oy), len[1], half[1]);
    const double dz = min_image(__dsub_rn(z, oz), len[2], half[2]);
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
    ql_bond<LT>(dx, dy, dz, r, l, re, im);
  }
  double sum = 0.0;
  if (bonds > 0) {
    const double inv = 1.0 / bonds;
#pragma unroll
    for (int m = 0; m < NM; m++) {
      if (m > l) break;
      const double a = f2_value(re[m]) * inv, b = f2_value(im[m]) * inv;
      sum += (m == 0 ? 1.0 : 2.0) * (a * a + b * b);
    }
  }
  q_out[i] = sqrt(sum * (4.0 * 3.14159265358979323846 / (2 * l + 1)));
}

// Deterministic mean: one block sums in a fixed order.
__global__ void __launch_bounds__(1024) k_sum(const double *q, int n, double *out) {
  __shared__ double part[1024];
  double a = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a += q[i];
  part[threadIdx.x] = a;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = part[0];
}

void launch_ql(const SysPtrs &p, int l, double rc, int stencil[3], double *per_particle, double *sum,
               cudaStream_t st) {
  QlCoef h;
  for (int m = 0; m <= QL_LMAX; m++) {
    h.neg_diag[m] = f2_of(m > 0 ? -sqrt((2.0 * m + 1.0) / (2.0 * m)) : 0.0);
    h.first[m] = f2_of(sqrt(2.0 * m + 3.0));
    for (int ll = 0; ll <= QL_LMAX; ll++) {
      const double den = (double)ll * ll - (double)m * m;
      h.a[ll][m] = f2_of(den > 0 ? sqrt((4.0 * ll * ll - 1.0) / den) : 0.0);
      const double nb = (ll - 1.0) * (ll - 1.0) - (double)m * m;
      const double db = 4.0 * (ll - 1.0) * (ll - 1.0) - 1.0;
      h.b[ll][m] = f2_of((nb >= 0 && db > 0) ? sqrt(nb / db) : 0.0);
    }
  }
  cudaMemcpyToSymbolAsync(c_ql, &h, sizeof(h), 0, cudaMemcpyHostToDevice, st);
  Stencil s{{stencil[0], stencil[1], stencil[2]}};
  const float cut = (float)rc + 1e-3f;
  const int blocks = (p.n + 127) / 128;
  const dim3 grid(blocks > 0 ? blocks : 1);
  if (l == 6) k_ql<6><<<grid, 128, 0, st>>>(p, s, l, rc, cut * cut, per_particle);
  else if (l == 4) k_ql<4><<<grid, 128, 0, st>>>(p, s, l, rc, cut * cut, per_particle);
  else k_ql<0><<<grid, 128, 0, st>>>(p, s, l, rc, cut * cut, per_particle);
  k_sum<<<1, 1024, 0, st>>>(per_particle, p.n, sum);
}

}  // namespace hsmc
