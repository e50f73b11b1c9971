// Internal interface between the C ABI (api.cu) and the kernel files.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

struct hsmc_ctx;

namespace hsmc {

// Pointers every kernel of one system needs.  All are device addresses that
// stay fixed for the life of a context, so captured CUDA graphs stay valid.
struct SysPtrs {
  double *pos;         // N x 4 doubles: (id, x, y, z), the reference's layout
  int *cnt[2];         // per-cell particle counts, one array per layout
  Slot *slot[2];       // per-cell slots, capacity `cap`, one array per layout
  Box *box;            // box and cell grid
  DevState *st;        // counters, parameters, status
  uint32_t *trace;     // trace records (12 words each) or nullptr
  unsigned long long trace_cap;
  int n;               // particles
  int cap;             // slots per cell
  int ncell_alloc;     // cells allocated per layout
  // Occupancy order of a single system's colour passes (batches: nullptr).
  // olist: per colour c, entries [c * ncell_alloc / 8, ...) list the colour's
  // non-empty cells, fullest first.  ocnt: words [32 c + n - 1] count the
  // cells of colour c holding n particles (n > 32 counts as 32), words
  // [256 + 32 c + n - 1] are the scatter's cursors, word 512 + c the number
  // of non-empty cells of colour c.
  int *olist;
  int *ocnt;
};

constexpr int kOrderWords = 520;  // words of SysPtrs::ocnt

// The replica holding flat index x, for batched launches over all replicas:
// the last r with start[r] <= x (start has n + 1 ascending entries).
__device__ __forceinline__ int find_rep(const int *start, int n, int x) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(start + mid) <= x) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// The grid shift of sweep s of replica rep: a uniform point of one cell
// (w = the cell edges), from 24-bit fractions of one Philox draw.
__device__ __forceinline__ void sweep_shift(uint64_t seed, uint32_t rep, unsigned long long s, const float w[3],
                                            float sh[3]) {
  const U32x4 rs = draw4(seed, rep << 8, 0u, s, TAG_SHIFT);
  sh[0] = __fmul_rn(__uint2float_rn(rs.x >> 8) * 5.9604644775390625e-08f, w[0]);
  sh[1] = __fmul_rn(__uint2float_rn(rs.y >> 8) * 5.9604644775390625e-08f, w[1]);
  sh[2] = __fmul_rn(__uint2float_rn(rs.z >> 8) * 5.9604644775390625e-08f, w[2]);
}

// The colour order of the eight passes of sweep s of replica rep: a
// Fisher-Yates shuffle driven by seven Philox words.
__device__ __forceinline__ void sweep_perm(uint64_t seed, uint32_t rep, unsigned long long s, int perm[8]) {
  for (int k = 0; k < 8; k++) perm[k] = k;
  const U32x4 ra = draw4(seed, rep << 8, 0u, s, TAG_PERM), rb = draw4(seed, (rep << 8) | 1u, 0u, s, TAG_PERM);
  const uint32_t r[7] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z};
  for (int k = 7; k >= 1; k--) {
    const int j = (int)__umulhi(r[7 - k], (unsigned)(k + 1));
    const int tmp = perm[k];
    perm[k] = perm[j];
    perm[j] = tmp;
  }
}

// The arrays of one layout.  A select, not an index: indexing the parameter
// struct by a runtime value would copy it to local memory.
__device__ __forceinline__ int *cnt_of(const SysPtrs &p, int layout) { return layout ? p.cnt[1] : p.cnt[0]; }
__device__ __forceinline__ Slot *slot_of(const SysPtrs &p, int layout) { return layout ? p.slot[1] : p.slot[0]; }

// vol_move (src/moves.c:83-153) in the reference's operation order, without
// contraction, shared by the volume-move kernels (sweep.cu) and the
// one-block sweep (sweep_small.cu) so that both make the same chain.
// The proposal: ln V' = ln V + (u - 1/2) dv_max, ratio V'/V, sf = ratio^(1/3).
__device__ __forceinline__ void vol_proposal(double vol, uint32_t r, double dv_max, double &vol_new, double &ratio,
                                             double &sf) {
  vol_new = exp(__dadd_rn(log(vol), __dmul_rn(centred_offset(r), dv_max)));
  ratio = __ddiv_rn(vol_new, vol);
  sf = pow(ratio, 1. / 3.);
}

// Whether the overlap scan of a volume move can be skipped: an expansion
// (sf > 1) scales every component of every pair's distance up, so it finds
// an overlap only where the configuration already holds a pair short of
// contact.  The chain itself leaves such pairs behind only as rounding: the
// rescale of an accepted volume move (x sf, and the box rebuilt from the
// density) can put a pair within a few ulp(L) below contact, where the
// reference's next scan, at a scale factor that close to 1, reports an
// overlap.  So the scan is skipped only for sf >= 1 + 2^-46 (L + 1), L the
// longest side (about 1e-12 at L = 100, far above that rounding); an
// expansion closer to 1, or sf = 1, is scanned.
__device__ __forceinline__ bool vol_scan_needed(double sf, const double len[3]) {
  double lmax = len[0] > len[1] ? len[0] : len[1];
  lmax = len[2] > lmax ? len[2] : lmax;
  return !(sf >= 1.0 + 1.4210854715202004e-14 * (lmax + 1.0));
}

// The acceptance bound exp(beta P (V - V') + (N + 1) ln(V'/V)).
__device__ __forceinline__ double vol_boltz(double pressure, double vol, double vol_new, int n, double ratio) {
  return exp(__dadd_rn(__dmul_rn(pressure, __dsub_rn(vol, vol_new)), __dmul_rn((double)(n + 1), log(ratio))));
}

// The box after an accepted volume move, rebuilt from the lattice counts
// and the new density as sim_box_init does (src/moves.c:128-132,
// src/sim_info.c:32-71), with the device grid re-derived for it (an even
// count per axis, edge >= 1 + margin, at most the allocated count).
// Returns false when the grid would have fewer than 4 cells per axis.
__device__ __forceinline__ bool vol_rebuild_box(const DevState *st, int n, double vol_new, double margin, Box &bx) {
  const double rho = n / vol_new;
  const double cell_vol = st->per_cell / rho;
  const double cell_size = pow(cell_vol, 1. / 3.);
  double lmax = 0.0;
  for (int d = 0; d < 3; d++) {
    const double len = st->cells[d] * cell_size;
    int nc = 2 * (int)floor(len / (2.0 * (1.0 + margin)));
    if (nc > st->nc_alloc[d]) nc = st->nc_alloc[d];
    if (nc < 4) return false;
    bx.len[d] = len;
    bx.half[d] = len / 2.0;
    bx.len32[d] = (float)len;
    bx.inv_w32[d] = (float)(nc / len);
    bx.w32[d] = (float)(len / nc);
    bx.nc[d] = nc;
    lmax = len > lmax ? len : lmax;
  }
  bx.ncell = bx.nc[0] * bx.nc[1] * bx.nc[2];
  bx.vol = st->cells[0] * st->cells[1] * st->cells[2] * cell_vol;
  bx.rho = rho;
  bx.band = (float)(5.9604644775390625e-08 * (48.0 * lmax + 16.0) + 1e-6);
  return true;
}

// api.cu: what other parts of the library see of a context
struct CtxView {
  SysPtrs sp;
  Box box;              // host copy of the current box
  cudaStream_t stream;  // the context's stream; calls are synchronous on it
  int num_sms;
  bool uploaded;        // a configuration is on the device and laid out
};
int ctx_view(::hsmc_ctx *ctx, CtxView *out);

// api.cu: device cell grid for a box (even count per axis, edge >= 1 + margin)
int make_box(const double len[3], double rho, Box &b, int &cap, double min_edge = 0.0);

// sweep.cu
void launch_build(const SysPtrs &p, long long sweep_offset, int num_sms, cudaStream_t s);
// After a sweep's build: each colour's non-empty cells listed fullest first
// (SysPtrs::olist), which the colour passes hand out to their warps.
void launch_order(const SysPtrs &p, cudaStream_t s);
// The same for the replicas of one cell capacity of a batch: a list per pass
// of (replica within the class, cell) pairs (olist, 2 ints each, stride
// entries per pass), counts in ocnt (kOrderWords ints); cstart: prefix sums
// of the replicas' cells, n_cells their total.
void launch_order_batch(const SysPtrs *reps, const int *cstart, int n_reps, long long n_cells, int *ocnt,
                        int *olist, int stride, cudaStream_t s);
// Flags an uploaded configuration whose ids are not 0..N-1 (ST_BAD_ID) or
// with a coordinate outside [0, L] (ST_OUT_OF_BOX; NaN included).
void launch_check_config(const SysPtrs &p, cudaStream_t s);
void launch_move_pass(const SysPtrs &p, int pass, int group, bool trace, int grid, cudaStream_t s);
void launch_advance(const SysPtrs &p, int n_sweeps, cudaStream_t s);
void launch_opt_step(const SysPtrs &p, int j, int n_samples, unsigned long long sweep_moves, double part_target,
                     double vol_target, bool npt, cudaStream_t s);
void launch_fill_u32(uint32_t *p, int n, uint32_t v, cudaStream_t s);
void launch_volume_move(const SysPtrs &p, long long sweep_offset, double margin, cudaStream_t s);
void launch_volume_scan(const SysPtrs &p, cudaStream_t s);
int move_pass_grid(int group, int cap, int ncell_alloc, int num_sms);
bool move_pass_fits(int group, int cap);  // its shared memory fits a block on this device
void prepare_move_pass();                 // allow each variant its shared memory (current device)
// dataflow sweep (all eight passes, cooperative launch); prog holds one
// progress word per 2x2x2 region (ncell_alloc / 8)
int move_flow_grid(int group, int cap, int ncell_alloc, int num_sms);
cudaError_t launch_move_flow(const SysPtrs &p, uint32_t *prog, int group, bool trace, int grid, cudaStream_t s);

// batched replicas: reps is a device array of n_reps SysPtrs
// nstart / gstart: prefix sums over replicas of particles / active cells
// (cells of one colour); launches cover all of them in one flat grid.
void launch_build_batch(const SysPtrs *reps, const int *nstart, int n_reps, int tot_n, long long sweep_offset,
                        cudaStream_t s);
// one launch per cell capacity: reps / gstart / ids over the replicas of
// that capacity (ids: their index in the batch); pools non-null clears the
// other layout of the pooled counts on pass 0; olist / ocnt non-null: the
// class's occupancy lists (launch_order_batch), which the pass follows
void launch_move_pass_batch(const SysPtrs *reps, const int *gstart, const int *ids, int n_reps, int tot_groups,
                            int cap, int pass, int group, int *cnt_pool0, int *cnt_pool1, long long pool_cells,
                            int *olist, int *ocnt, cudaStream_t s);
void launch_advance_batch(const SysPtrs *reps, int n_reps, int n_sweeps, cudaStream_t s);
void launch_pair_hist_batch(const SysPtrs *reps, int n_reps, int max_n, double bin, double rmax, int nbins,
                            unsigned long long *counts, cudaStream_t s);

// cluster.cu: n_moves geometric cluster moves in one cooperative launch of
// `grid` blocks, each followed by a rebuild of the current layout
// (ctr[3] must be zero at launch)
struct ClusterJob {
  int *queue;                // n entries: the cluster, level by level
  uint32_t *mark;            // n words: epoch of the move that took each particle
  uint32_t *ctr;             // [0..2] particles found per level (rotating), [3] barrier arrivals
  long long *size_out;       // n_moves cluster sizes
  double *drawn;             // 5 x n_moves: pivot x, y, z, axis, seed particle; or nullptr
  double pivot[3];           // used when `given` (then n_moves = 1)
  double sint;               // sin(M_PI) of the host libm (its cos(M_PI) is -1)
  unsigned long long seq;    // index of the first move in the context's stream
  uint32_t epoch;            // first move's epoch; epoch .. epoch + n_moves - 1 match no mark
  int axis, seed_id, given;
};
// grid 0: the whole system fits one block's shared memory (k_cluster_small);
// its launch leaves the cell layout to the caller
int cluster_grid(int n, int ncell, int num_sms);
cudaError_t launch_cluster(const SysPtrs &p, const ClusterJob &job, int n_moves, int grid, int ncell,
                           cudaStream_t s);

// sweep_small.cu: every sweep of a call in one block with the system in
// shared memory (0 bytes: the system does not fit; ncell the allocated
// grid); the same chain as the pass-barrier schedule, with one volume move
// per sweep when npt.  The launch leaves the device cell layouts stale.
size_t sweep_small_smem(int n, int ncell, int cap);
bool prepare_sweep_small(size_t smem);
void launch_sweep_small(const SysPtrs &p, int n_sweeps, bool npt, bool cavity, double margin, size_t smem,
                        cudaStream_t s);

// cavity.cu: the cavity trials of sweep sweep_base + offset (trace: 8 words
// per trial or nullptr), and psi at n distances
void launch_cavity(const SysPtrs &p, long long sweep_offset, uint32_t *trace, long long trace_cap, cudaStream_t s);
void launch_cavity_psi(const SysPtrs &p, const double *x, int n, double *out, cudaStream_t s);

// observables.cu
void launch_pair_hist(const SysPtrs &p, double bin, double rmax, int nbins, unsigned long long *counts,
                      int stencil[3], cudaStream_t s, const double *thr = nullptr);
void launch_scaled_scan(const SysPtrs &p, const double *sf, int n_sf, int stencil[3], cudaStream_t s);
void launch_widom(const SysPtrs &p, long long n, unsigned long long seq, const double *pos_in, uint8_t *ov_out,
                  cudaStream_t s);
void launch_overlap_replay(const SysPtrs &p, const int *ids, const double *pos_in, int n, uint8_t *ov_out,
                           cudaStream_t s);
void launch_ql(const SysPtrs &p, int l, double rc, int stencil[3], double *per_particle, double *sum,
               cudaStream_t s);

}  // namespace hsmc
