// C ABI of the GB300 hard-sphere Monte Carlo engine (include/hsmc_gpu.h).
//
// A context owns one system on the current device: positions in the
// reference's double[N][4] layout, two fixed-capacity cell layouts that the
// sweeps alternate between, the box, and a device state block with the
// counters and the random-stream position.  Sweeps run as CUDA graphs of
// (build + 8 move passes) x S sweeps; every call is synchronous on the
// context's stream.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/hsmc_gpu.h"
#include "engine.cuh"

using namespace hsmc;

namespace {

constexpr int kGraphSweeps = 8;
constexpr int kDefaultLanes = 2;  // lanes per active cell in a move pass
constexpr int kFastBins = 2048;   // pair counts with bin thresholds (observables.cu FAST_BINS)

struct Scratch {
  void *ptr = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
};

}  // namespace

struct hsmc_ctx {
  hsmc_params prm{};
  int n = 0;
  int num_sms = 0;
  int group = 8;
  int pass_grid = 1;
  cudaStream_t stream = nullptr;
  SysPtrs sp{};
  Box hbox{};
  unsigned long long sweep_base = 1;  // host mirror of DevState::sweep_base
  unsigned long long widom_seq = 0;
  bool uploaded = false;
  bool profiling = false;
  cudaGraphExec_t graph = nullptr;      // NVT: kGraphSweeps x (build + 8 passes) + advance
  cudaGraphExec_t graph_npt = nullptr;  // NpT: the same plus one volume move per sweep
  double margin = 0.0;                  // grid margin over 1 of the cell edge
  cudaEvent_t ev_start = nullptr, ev_stop = nullptr;
  std::vector<cudaEvent_t> ev_pass;
  double last_total_ms = 0.0, last_move_ms = 0.0;
  int last_move_launches = 0;
  Scratch hist, qbuf, flags, qpos, qids, trace;
  // bin thresholds of the last pair-count call (hsmc_pair_thresholds)
  Scratch thr;
  std::vector<double> thr_host;
  double thr_dr = 0.0, thr_rmax = 0.0;
  int thr_nbins = 0;
  // dataflow schedule: one cooperative launch per sweep, progress words per
  // 2x2x2 region; `flow_graph` records whether such launches capture
  bool flow = false;
  int flow_grid = 0;
  int flow_graph = -1;  // -1 untested, 0 no, 1 yes
  uint32_t *prog = nullptr;
  // schedule 3: each colour's non-empty cells listed fullest first
  // (SysPtrs::olist points here while that schedule is in use)
  int *olist = nullptr;
  // cluster moves: queue (N ints), marks (N words), counters, per-move output
  Scratch cl_queue, cl_mark, cl_ctr, cl_out;
  unsigned long long cluster_seq = 0;  // cluster moves drawn from the stream so far
  uint32_t cl_epoch = 0;               // epoch of the last move (marks hold older ones)
  int cl_grid = -1;  // -1 not chosen yet, 0 the one-block shared-memory kernel
  // one-block schedule (sweep_small.cu): shared memory it needs (0: the
  // system does not fit) and whether it is the schedule in use
  size_t small_smem = 0;
  bool small = false;
  // cavity sampling: on when the context was created with cavity_pcav > 0
  bool cavity = false;
  Scratch cav_trace;
  long long cav_trace_cap = 0;
};

// ----------------------------------------------------------------- helpers

// Progress words of the dataflow schedule: "every pass of the sweep before
// sweep_base is done", written whenever the sweep index is set.
static void reset_progress(hsmc_ctx *ctx) {
  launch_fill_u32(ctx->prog, ctx->sp.ncell_alloc / 8 + 1, (uint32_t)(ctx->sweep_base * 8ull), ctx->stream);
}


int hsmc::ctx_view(hsmc_ctx *ctx, CtxView *out) {
  if (!ctx || !out) return HSMC_ERR_INVALID_ARG;
  out->sp = ctx->sp;
  out->box = ctx->hbox;
  out->stream = ctx->stream;
  out->num_sms = ctx->num_sms;
  out->uploaded = ctx->uploaded;
  return HSMC_OK;
}

static int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return HSMC_OK;
  fprintf(stderr, "hsmc_gpu: CUDA error %s\n", cudaGetErrorString(e));
  return HSMC_ERR_CUDA;
}

#define HSMC_CUDA(call)                      \
  do {                                       \
    cudaError_t e_ = (call);                 \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

static int status_to_code(int st) {
  if (st & ST_BAD_ID) return HSMC_ERR_INVALID_ARG;
  if (st & ST_CELL_OVERFLOW) return HSMC_ERR_CELL_OVERFLOW;
  if (st & ST_BAD_BIN) return HSMC_ERR_BAD_BIN;
  if (st & ST_OUT_OF_BOX) return HSMC_ERR_OUT_OF_BOX;
  if (st & ST_TRACE_FULL) return HSMC_ERR_INVALID_ARG;
  if (st & ST_BAD_CELL) return HSMC_ERR_CELL_OVERFLOW;
  if (st & (ST_FLOW_TIMEOUT | ST_CLUSTER_TIMEOUT)) return HSMC_ERR_TIMEOUT;
  if (st & ST_CAVITY_RANGE) return HSMC_ERR_CAVITY_RANGE;
  return HSMC_OK;
}

// Cell grid for a box: an even number of cells per axis, each edge at least
// 1 + margin, the margin covering single-precision rounding of coordinates
// up to the box length.
int hsmc::make_box(const double len[3], double rho, Box &b, int &cap, double min_edge) {
  double lmax = len[0];
  for (int d = 1; d < 3; d++) lmax = len[d] > lmax ? len[d] : lmax;
  const double u = 5.9604644775390625e-08;  // 2^-24
  const double margin = u * (64.0 * lmax + 64.0);
  double wmax = 0.0;
  const double wmin = min_edge > 1.0 + margin ? min_edge : 1.0 + margin;
  for (int d = 0; d < 3; d++) {
    int nc = 2 * (int)std::floor(len[d] / (2.0 * wmin));
    if (nc < 4) return HSMC_ERR_CELL_TOO_SMALL;
    b.len[d] = len[d];
    b.half[d] = len[d] / 2.0;
    b.len32[d] = (float)len[d];
    b.inv_w32[d] = (float)(nc / len[d]);
    b.w32[d] = (float)(len[d] / nc);
    b.nc[d] = nc;
    const double w = len[d] / nc;
    wmax = w > wmax ? w : wmax;
  }
  b.ncell = b.nc[0] * b.nc[1] * b.nc[2];
  b.vol = len[0] * len[1] * len[2];
  b.rho = rho;
  // |error of r^2| of the screen: about 3.5 * 2^-24 * (11 L + 2); doubled.
  b.band = (float)(u * (48.0 * lmax + 16.0) + 1e-6);
  b.pad = 0;
  // Points at mutual distance >= 1 in a cube of edge w: at most 8 below
  // 2/sqrt(3), at most 14 below sqrt(2).
  cap = wmax < 1.15 ? 8 : (wmax < 1.41 ? 16 : 32);
  return HSMC_OK;
}

static int stencil_for(const Box &b, double cut, int k[3]) {
  for (int d = 0; d < 3; d++) {
    const double w = b.len[d] / b.nc[d];
    int kk = (int)std::ceil((cut + 1e-3) / w);
    if (kk < 1) kk = 1;
    k[d] = (2 * kk + 1 >= b.nc[d]) ? -1 : kk;
  }
  return 0;
}

static int read_state(hsmc_ctx *ctx, DevState &out) {
  HSMC_CUDA(cudaMemcpyAsync(&out, ctx->sp.st, sizeof(DevState), cudaMemcpyDeviceToHost, ctx->stream));
  HSMC_CUDA(cudaStreamSynchronize(ctx->stream));
  return HSMC_OK;
}

static int check_kernels(hsmc_ctx *ctx) {
  HSMC_CUDA(cudaGetLastError());
  HSMC_CUDA(cudaStreamSynchronize(ctx->stream));
  return HSMC_OK;
}

// Device time of an observable call's kernels, for hsmc_gpu_last_timing:
// events on the context's stream around the launches, read once the call
// has synchronised.
static void timing_begin(hsmc_ctx *ctx) { cudaEventRecord(ctx->ev_start, ctx->stream); }
static void timing_end(hsmc_ctx *ctx) { cudaEventRecord(ctx->ev_stop, ctx->stream); }
static void timing_read(hsmc_ctx *ctx) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop) == cudaSuccess) ctx->last_total_ms = ms;
  ctx->last_move_ms = 0.0;
  ctx->last_move_launches = 0;
}

static void clear_counters_async(hsmc_ctx *ctx) {
  // acc .. vol_acc, trace_count, widom_ok, scan_mask: one contiguous run
  cudaMemsetAsync(&ctx->sp.st->acc, 0, offsetof(DevState, dr_max) - offsetof(DevState, acc), ctx->stream);
}

// ------------------------------------------------------------------- ABI

extern "C" {

const char *hsmc_gpu_strerror(int status) {
  switch (status) {
    case HSMC_OK: return "ok";
    case HSMC_ERR_INVALID_ARG: return "ERROR: invalid argument";
    case HSMC_ERR_CUDA: return "ERROR: CUDA runtime failure";
    case HSMC_ERR_NO_DEVICE: return "ERROR: no sm_103 GPU available";
    case HSMC_ERR_CELL_OVERFLOW: return "ERROR: More than the allowed number of particles in one cell";
    case HSMC_ERR_CELL_TOO_SMALL:
      return "ERROR: size of cells in cell list is smaller than the size of the particles";
    case HSMC_ERR_BAD_BIN: return "ERROR: pair distance outside the histogram (overlapping configuration)";
    case HSMC_ERR_TIMEOUT: return "ERROR: device wait timed out";
    case HSMC_ERR_OUT_OF_BOX: return "ERROR: coordinate outside the simulation box";
    case HSMC_ERR_OVERLAP: return "Overlap in the initial configuration";
    case HSMC_ERR_CAVITY_RANGE: return "Error, the cavities are too close or too far apart!";
    default: return "ERROR: unknown status";
  }
}

int hsmc_gpu_create(const hsmc_params *prm, hsmc_ctx **out) {
  if (!prm || !out) return HSMC_ERR_INVALID_ARG;
  *out = nullptr;
  if (prm->n_particles <= 0 || !(prm->box[0] > 0) || !(prm->box[1] > 0) || !(prm->box[2] > 0) ||
      !(prm->dr_max >= 0) || !(prm->dv_max >= 0))
    return HSMC_ERR_INVALID_ARG;
  for (int d = 0; d < 3; d++)
    if (!(prm->dr_max < prm->box[d])) return HSMC_ERR_INVALID_ARG;
  // the device re-derives an NpT grid with the standard edge only
  if (!(prm->min_cell_edge >= 0.0) || (prm->min_cell_edge > 0.0 && prm->pressure > 0)) return HSMC_ERR_INVALID_ARG;
  const bool cavity = prm->cavity_pcav > 0;
  if (!(prm->cavity_pcav >= 0.0) || prm->cavity_pcav > 1.0) return HSMC_ERR_INVALID_ARG;
  if (cavity && (prm->pressure > 0 || prm->n_particles < 3 || !(prm->cavity_mindr >= 0.0) ||
                 !(prm->cavity_maxdr > prm->cavity_mindr)))
    return HSMC_ERR_INVALID_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return HSMC_ERR_NO_DEVICE;
  cudaDeviceProp p{};
  if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) return HSMC_ERR_NO_DEVICE;
  if (!(p.major == 10 && p.minor == 3)) {
    fprintf(stderr, "hsmc_gpu: device %s is sm_%d%d; this build targets sm_103a\n", p.name, p.major, p.minor);
    return HSMC_ERR_NO_DEVICE;
  }
  Box b{};
  int cap = 8;
  const double rho = prm->n_particles / (prm->box[0] * prm->box[1] * prm->box[2]);
  int e = make_box(prm->box, prm->rho > 0 ? prm->rho : rho, b, cap, prm->min_cell_edge);
  if (e) return e;
  // NpT boxes change: cells are allocated for a box 25% longer per side, and
  // the grid margin is fixed for that largest box.
  Box balloc = b;
  int cap_alloc = cap;
  if (prm->pressure > 0) {
    const double grown[3] = {prm->box[0] * 1.25, prm->box[1] * 1.25, prm->box[2] * 1.25};
    if ((e = make_box(grown, b.rho, balloc, cap_alloc))) return e;
  }
  if (prm->cell_capacity > 0) {
    if (prm->cell_capacity > 32) return HSMC_ERR_INVALID_ARG;
    cap = prm->cell_capacity <= 8 ? 8 : (prm->cell_capacity <= 16 ? 16 : 32);
  }
  // the two cavities may overlap each other: one more sphere than geometry allows
  if (cavity && cap < 16) cap = 16;

  prepare_move_pass();
  hsmc_ctx *ctx = new hsmc_ctx();
  ctx->prm = *prm;
  ctx->n = prm->n_particles;
  ctx->num_sms = p.multiProcessorCount;
  ctx->hbox = b;
  // A system with more active cells than one wave of 2-lane groups runs
  // each group through several cells a pass.  There 8 lanes a cell shorten
  // each cell's chain more than the extra waves cost, and the occupancy
  // order (schedule 3) takes the empty cells out of the waves and gives each
  // warp cells of one occupancy (measured at N = 1,048,576: 8 lanes 1.27x the
  // trial moves/s of 2, the occupancy order another 1.12x).  Within one wave
  // the grid order is faster: the two order launches and the scattered
  // cells cost more there than the shorter trial rounds save.
  // hsmc_gpu_autotune times every choice on the live system.
  const long long active_cells = (long long)b.ncell / 8;
  const bool beyond_wave = active_cells > 4ll * p.multiProcessorCount * (128 / kDefaultLanes);
  switch (prm->lanes_per_cell) {
    case 0:
      ctx->group = (beyond_wave && move_pass_fits(8, cap)) ? 8 : kDefaultLanes;
      break;
    case 1: case 2: case 4: case 8: ctx->group = prm->lanes_per_cell; break;
    default: delete ctx; return HSMC_ERR_INVALID_ARG;
  }
  if (!move_pass_fits(ctx->group, cap)) {  // one lane per cell with 32-slot cells
    delete ctx;
    return HSMC_ERR_INVALID_ARG;
  }
  SysPtrs &sp = ctx->sp;
  sp.n = ctx->n;
  sp.cap = cap;
  sp.ncell_alloc = balloc.ncell;
  {
    double lmax = balloc.len[0];
    for (int d = 1; d < 3; d++) lmax = balloc.len[d] > lmax ? balloc.len[d] : lmax;
    ctx->margin = 5.9604644775390625e-08 * (64.0 * lmax + 64.0);
  }
  auto fail = [&](cudaError_t err) {
    hsmc_gpu_destroy(ctx);
    return cuda_status(err);
  };
  cudaError_t ce;
  if ((ce = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(ce);
  if ((ce = cudaMalloc(&sp.pos, sizeof(double) * 4 * (size_t)ctx->n)) != cudaSuccess) return fail(ce);
  for (int l = 0; l < 2; l++) {
    if ((ce = cudaMalloc(&sp.cnt[l], sizeof(int) * (size_t)sp.ncell_alloc)) != cudaSuccess) return fail(ce);
    if ((ce = cudaMalloc(&sp.slot[l], sizeof(Slot) * (size_t)sp.ncell_alloc * cap)) != cudaSuccess) return fail(ce);
    if ((ce = cudaMemset(sp.cnt[l], 0, sizeof(int) * (size_t)sp.ncell_alloc)) != cudaSuccess) return fail(ce);
  }
  if ((ce = cudaMalloc(&ctx->olist, sizeof(int) * (size_t)sp.ncell_alloc)) != cudaSuccess) return fail(ce);
  sp.olist = beyond_wave ? ctx->olist : nullptr;
  if ((ce = cudaMalloc(&sp.ocnt, sizeof(int) * (size_t)kOrderWords)) != cudaSuccess) return fail(ce);
  if ((ce = cudaMemset(sp.ocnt, 0, sizeof(int) * (size_t)kOrderWords)) != cudaSuccess) return fail(ce);
  if ((ce = cudaMalloc(&sp.box, sizeof(Box))) != cudaSuccess) return fail(ce);
  if ((ce = cudaMalloc(&sp.st, sizeof(DevState))) != cudaSuccess) return fail(ce);
  if ((ce = cudaMemcpy(sp.box, &b, sizeof(Box), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(ce);
  DevState s0{};
  s0.sweep_base = ctx->sweep_base;
  s0.dr_max = prm->dr_max;
  s0.dv_max = prm->dv_max;
  s0.pressure = prm->pressure;
  s0.seed = prm->seed;
  s0.per_cell = prm->lattice_type == 1 ? 1 : 4;
  s0.flow_hold = -1;
  if (cavity) {
    s0.frozen = 2;
    const long long k = std::llround((double)prm->n_particles * prm->cavity_pcav);
    s0.cav_trials = (int)(k < 1 ? 1 : k);
    s0.cav_min = prm->cavity_mindr;
    s0.cav_max = prm->cavity_maxdr;
    s0.cav_r2min = hsmc_cavity_r2_at_least(prm->cavity_mindr);
    s0.cav_r2max = hsmc_cavity_r2_at_most(prm->cavity_maxdr);
    hsmc_cavity_coeffs(prm->rho > 0 ? prm->rho : rho, &s0.psi);
  }
  for (int d = 0; d < 3; d++) {
    s0.cells[d] = prm->cells[d];
    s0.nc_alloc[d] = balloc.nc[d];
  }
  if ((ce = cudaMemcpy(sp.st, &s0, sizeof(DevState), cudaMemcpyHostToDevice)) != cudaSuccess) return fail(ce);
  if ((ce = cudaEventCreate(&ctx->ev_start)) != cudaSuccess) return fail(ce);
  if ((ce = cudaEventCreate(&ctx->ev_stop)) != cudaSuccess) return fail(ce);
  ctx->pass_grid = move_pass_grid(ctx->group, cap, sp.ncell_alloc, ctx->num_sms);
  if ((ce = cudaMalloc(&ctx->prog, sizeof(uint32_t) * (size_t)(sp.ncell_alloc / 8 + 1))) != cudaSuccess)
    return fail(ce);
  ctx->flow = false;  // one launch per pass unless hsmc_gpu_set_schedule or the autotuner picks the dataflow sweep
  ctx->cavity = cavity;
  // a system that fits one block's shared memory (at the largest grid its
  // box may reach) runs its sweeps there
  {
    const size_t sm = sweep_small_smem(ctx->n, balloc.ncell, cap);
    if (sm > 0 && prepare_sweep_small(sm)) ctx->small_smem = sm;
    cudaGetLastError();
  }
  // the default where it measured faster than one launch per pass: at most
  // 128 active cells per pass (up to about 1000 spheres); the autotuner
  // tries it wherever it fits
  ctx->small = ctx->small_smem > 0 && b.ncell / 8 <= 128;
  *out = ctx;
  return HSMC_OK;
}

void hsmc_gpu_destroy(hsmc_ctx *ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  if (ctx->graph_npt) cudaGraphExecDestroy(ctx->graph_npt);
  SysPtrs &sp = ctx->sp;
  cudaFree(sp.pos);
  for (int l = 0; l < 2; l++) {
    cudaFree(sp.cnt[l]);
    cudaFree(sp.slot[l]);
  }
  cudaFree(ctx->olist);
  cudaFree(sp.ocnt);
  cudaFree(sp.box);
  cudaFree(sp.st);
  cudaFree(ctx->prog);
  ctx->hist.release();
  ctx->qbuf.release();
  ctx->flags.release();
  ctx->qpos.release();
  ctx->qids.release();
  ctx->trace.release();
  ctx->thr.release();
  ctx->cl_queue.release();
  ctx->cl_mark.release();
  ctx->cl_ctr.release();
  ctx->cl_out.release();
  ctx->cav_trace.release();
  if (ctx->ev_start) cudaEventDestroy(ctx->ev_start);
  if (ctx->ev_stop) cudaEventDestroy(ctx->ev_stop);
  for (cudaEvent_t e : ctx->ev_pass) cudaEventDestroy(e);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

// The configuration is checked on the device after the copy (ids 0..N-1,
// coordinates in [0, L]); a configuration that fails leaves the context
// without one (the sweep calls refuse to run until an upload succeeds).
int hsmc_gpu_upload_config(hsmc_ctx *ctx, const double (*conf)[4], int n) {
  if (!ctx || !conf || n != ctx->n) return HSMC_ERR_INVALID_ARG;
  ctx->uploaded = false;
  SysPtrs &sp = ctx->sp;
  HSMC_CUDA(cudaMemcpyAsync(sp.pos, conf, sizeof(double) * 4 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  HSMC_CUDA(cudaMemsetAsync(&sp.st->status, 0, sizeof(int), ctx->stream));
  launch_check_config(sp, ctx->stream);
  int e = check_kernels(ctx);
  if (e) return e;
  DevState s;
  if ((e = read_state(ctx, s))) return e;
  if (s.status) return status_to_code(s.status);
  for (int l = 0; l < 2; l++)
    HSMC_CUDA(cudaMemsetAsync(sp.cnt[l], 0, sizeof(int) * (size_t)sp.ncell_alloc, ctx->stream));
  launch_build(sp, -1, ctx->num_sms, ctx->stream);
  reset_progress(ctx);
  e = check_kernels(ctx);
  if (e) return e;
  if ((e = read_state(ctx, s))) return e;
  if (s.status) return status_to_code(s.status);
  ctx->uploaded = true;
  return HSMC_OK;
}

int hsmc_gpu_download_config(hsmc_ctx *ctx, double (*conf)[4], int n) {
  if (!ctx || !conf || n != ctx->n) return HSMC_ERR_INVALID_ARG;
  HSMC_CUDA(cudaMemcpyAsync(conf, ctx->sp.pos, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
  HSMC_CUDA(cudaStreamSynchronize(ctx->stream));
  return HSMC_OK;
}

int hsmc_gpu_set_step(hsmc_ctx *ctx, double dr_max, double dv_max) {
  if (!ctx || !(dr_max >= 0) || !(dv_max >= 0)) return HSMC_ERR_INVALID_ARG;
  // A displacement of at most dr_max/2 per axis must stay within one periodic
  // wrap (apply_pbc wraps once).
  for (int d = 0; d < 3; d++)
    if (!(dr_max < ctx->hbox.len[d])) return HSMC_ERR_INVALID_ARG;
  ctx->prm.dr_max = dr_max;
  ctx->prm.dv_max = dv_max;
  double v[2] = {dr_max, dv_max};
  HSMC_CUDA(cudaMemcpyAsync(&ctx->sp.st->dr_max, v, sizeof(v), cudaMemcpyHostToDevice, ctx->stream));
  HSMC_CUDA(cudaStreamSynchronize(ctx->stream));
  return HSMC_OK;
}

int hsmc_gpu_set_profiling(hsmc_ctx *ctx, int on) {
  if (!ctx) return HSMC_ERR_INVALID_ARG;
  ctx->profiling = on != 0;
  return HSMC_OK;
}

int hsmc_gpu_last_timing(hsmc_ctx *ctx, double *total_ms, double *move_kernel_ms, int *move_launches) {
  if (!ctx) return HSMC_ERR_INVALID_ARG;
  if (total_ms) *total_ms = ctx->last_total_ms;
  if (move_kernel_ms) *move_kernel_ms = ctx->last_move_ms;
  if (move_launches) *move_launches = ctx->last_move_launches;
  return HSMC_OK;
}

// The eight passes of one sweep: one dataflow launch, or the occupancy
// order of the cells and eight launches with a kernel boundary after each
// colour.
static cudaError_t enqueue_moves(hsmc_ctx *ctx, bool trace) {
  if (ctx->flow) return launch_move_flow(ctx->sp, ctx->prog, ctx->group, trace, ctx->flow_grid, ctx->stream);
  if (ctx->sp.olist) launch_order(ctx->sp, ctx->stream);
  for (int k = 0; k < 8; k++) launch_move_pass(ctx->sp, k, ctx->group, trace, ctx->pass_grid, ctx->stream);
  return cudaSuccess;
}

// The cavity stage of a sweep (cavity.cu), after its colour passes.
static void enqueue_cavity(hsmc_ctx *ctx, long long offset) {
  if (ctx->cavity)
    launch_cavity(ctx->sp, offset, ctx->cav_trace_cap > 0 ? (uint32_t *)ctx->cav_trace.ptr : nullptr,
                  ctx->cav_trace_cap, ctx->stream);
}

static cudaError_t enqueue_sweep(hsmc_ctx *ctx, long long offset, bool trace, bool npt) {
  launch_build(ctx->sp, offset, ctx->num_sms, ctx->stream);
  cudaError_t e = enqueue_moves(ctx, trace);
  if (npt) launch_volume_move(ctx->sp, offset, ctx->margin, ctx->stream);
  enqueue_cavity(ctx, offset);
  return e;
}

static int ensure_graph(hsmc_ctx *ctx, bool npt) {
  cudaGraphExec_t &exec = npt ? ctx->graph_npt : ctx->graph;
  if (exec) return HSMC_OK;
  cudaGraph_t g = nullptr;
  HSMC_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t le = cudaSuccess;
  for (int s = 0; s < kGraphSweeps && le == cudaSuccess; s++) le = enqueue_sweep(ctx, s, false, npt);
  launch_advance(ctx->sp, kGraphSweeps, ctx->stream);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
  if (le != cudaSuccess || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (ctx->flow) {  // cooperative launches do not capture here: launch sweeps directly
      ctx->flow_graph = 0;
      return HSMC_OK;
    }
    return cuda_status(le != cudaSuccess ? le : e);
  }
  e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    exec = nullptr;
    cudaGetLastError();
    if (ctx->flow) {
      ctx->flow_graph = 0;
      return HSMC_OK;
    }
    return cuda_status(e);
  }
  if (ctx->flow) ctx->flow_graph = 1;
  return HSMC_OK;
}

// Rebuilds the layout of the last sweep in place (after volume moves the
// positions no longer match it), so observables see a consistent layout.
static void rebuild_current_layout(hsmc_ctx *ctx) {
  const int layout = (int)((ctx->sweep_base - 1) & 1ull);
  cudaMemsetAsync(ctx->sp.cnt[layout], 0, sizeof(int) * (size_t)ctx->sp.ncell_alloc, ctx->stream);
  launch_build(ctx->sp, -1, ctx->num_sms, ctx->stream);
}

static int run_sweeps(hsmc_ctx *ctx, int n_sweeps, bool trace, bool npt, uint64_t counters[6]) {
  if (!ctx || n_sweeps < 0) return HSMC_ERR_INVALID_ARG;
  if (!ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  clear_counters_async(ctx);
  HSMC_CUDA(cudaMemsetAsync(&ctx->sp.st->status, 0, sizeof(int), ctx->stream));
  ctx->last_move_ms = 0.0;
  ctx->last_move_launches = 0;
  if (ctx->small && !trace && !ctx->profiling && ctx->cav_trace_cap == 0) {
    // every sweep in one launch, then the device layouts rebuilt for the
    // last sweep (observables and the other schedules read them)
    HSMC_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
    if (n_sweeps > 0)
      launch_sweep_small(ctx->sp, n_sweeps, npt, ctx->cavity, ctx->margin, ctx->small_smem, ctx->stream);
    HSMC_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
    ctx->sweep_base += (unsigned long long)n_sweeps;
    if (n_sweeps > 0) {
      for (int l = 0; l < 2; l++)
        HSMC_CUDA(cudaMemsetAsync(ctx->sp.cnt[l], 0, sizeof(int) * (size_t)ctx->sp.ncell_alloc, ctx->stream));
      launch_build(ctx->sp, -1, ctx->num_sms, ctx->stream);
      reset_progress(ctx);
    }
    int e = check_kernels(ctx);
    if (e) return e;
    float ms = 0.f;
    HSMC_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
    ctx->last_total_ms = ms;
    DevState s;
    if ((e = read_state(ctx, s))) return e;
    if (npt) HSMC_CUDA(cudaMemcpy(&ctx->hbox, ctx->sp.box, sizeof(Box), cudaMemcpyDeviceToHost));
    if (counters) {
      const uint64_t moves = (uint64_t)ctx->n * (uint64_t)n_sweeps + s.cav_moves;
      counters[HSMC_CNT_MOVES] = moves;
      counters[HSMC_CNT_ACCEPTED] = s.acc + s.cav_acc;
      counters[HSMC_CNT_REJECTED] = moves - s.acc - s.cav_acc;
      counters[HSMC_CNT_VOL_MOVES] = s.vol_moves;
      counters[HSMC_CNT_VOL_ACCEPTED] = s.vol_acc;
      counters[HSMC_CNT_VOL_REJECTED] = s.vol_moves - s.vol_acc;
    }
    if (s.status) return status_to_code(s.status);
    return HSMC_OK;
  }
  bool direct = trace || ctx->profiling || ctx->cav_trace_cap > 0;  // graphs hold no trace buffers
  if (!direct) {
    int e = ensure_graph(ctx, npt);
    if (e) return e;
    if (ctx->flow && ctx->flow_graph == 0) direct = true;
  }
  const bool timing = ctx->profiling && !trace;
  if (timing) {
    const size_t need = 16 * (size_t)n_sweeps;
    while (ctx->ev_pass.size() < need) {
      cudaEvent_t ev;
      HSMC_CUDA(cudaEventCreate(&ev));
      ctx->ev_pass.push_back(ev);
    }
  }
  HSMC_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
  int done = 0;
  if (!direct) {
    while (n_sweeps - done >= kGraphSweeps) {
      HSMC_CUDA(cudaGraphLaunch(npt ? ctx->graph_npt : ctx->graph, ctx->stream));
      done += kGraphSweeps;
    }
  }
  const int rest = n_sweeps - done;
  const int per_sweep = ctx->flow ? 1 : 8;  // move-kernel launches per sweep
  for (int s = 0; s < rest; s++) {
    launch_build(ctx->sp, s, ctx->num_sms, ctx->stream);
    if (ctx->flow) {
      if (timing) HSMC_CUDA(cudaEventRecord(ctx->ev_pass[16 * s], ctx->stream));
      HSMC_CUDA(launch_move_flow(ctx->sp, ctx->prog, ctx->group, trace, ctx->flow_grid, ctx->stream));
      if (timing) HSMC_CUDA(cudaEventRecord(ctx->ev_pass[16 * s + 1], ctx->stream));
    } else {
      // timed as a whole: events between the passes would break the
      // programmatic dependent launches that overlap one pass's tail with
      // the next pass's start, so the eight passes are bracketed together
      if (ctx->sp.olist) launch_order(ctx->sp, ctx->stream);
      if (timing) HSMC_CUDA(cudaEventRecord(ctx->ev_pass[16 * s], ctx->stream));
      for (int k = 0; k < 8; k++) launch_move_pass(ctx->sp, k, ctx->group, trace, ctx->pass_grid, ctx->stream);
      if (timing) HSMC_CUDA(cudaEventRecord(ctx->ev_pass[16 * s + 1], ctx->stream));
    }
    if (npt) launch_volume_move(ctx->sp, s, ctx->margin, ctx->stream);
    enqueue_cavity(ctx, s);
  }
  if (rest > 0) launch_advance(ctx->sp, rest, ctx->stream);
  HSMC_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
  ctx->sweep_base += (unsigned long long)n_sweeps;
  // volume and cavity moves leave the last layout behind the positions
  if ((npt || ctx->cavity) && n_sweeps > 0) rebuild_current_layout(ctx);
  int e = check_kernels(ctx);
  if (e) return e;
  float ms = 0.f;
  HSMC_CUDA(cudaEventElapsedTime(&ms, ctx->ev_start, ctx->ev_stop));
  ctx->last_total_ms = ms;
  if (timing) {
    double sum = 0.0;
    for (int s = 0; s < rest; s++) {
      float t = 0.f;
      HSMC_CUDA(cudaEventElapsedTime(&t, ctx->ev_pass[16 * s], ctx->ev_pass[16 * s + 1]));
      sum += t;
    }
    ctx->last_move_ms = sum;
    ctx->last_move_launches = per_sweep * rest;
  }
  DevState s;
  if ((e = read_state(ctx, s))) return e;
  if (npt) {
    HSMC_CUDA(cudaMemcpy(&ctx->hbox, ctx->sp.box, sizeof(Box), cudaMemcpyDeviceToHost));
  }
  if (counters) {
    const uint64_t moves = (uint64_t)ctx->n * (uint64_t)n_sweeps + s.cav_moves;
    counters[HSMC_CNT_MOVES] = moves;
    counters[HSMC_CNT_ACCEPTED] = s.acc + s.cav_acc;
    counters[HSMC_CNT_REJECTED] = moves - s.acc - s.cav_acc;
    counters[HSMC_CNT_VOL_MOVES] = s.vol_moves;
    counters[HSMC_CNT_VOL_ACCEPTED] = s.vol_acc;
    counters[HSMC_CNT_VOL_REJECTED] = s.vol_moves - s.vol_acc;
  }
  if (s.status && !(trace && s.status == ST_TRACE_FULL)) return status_to_code(s.status);
  return HSMC_OK;
}

// Enqueues n_sweeps ordinary sweeps on the production path (one block, or
// graphs of 8 sweeps and single sweeps after them) without waiting for
// them: the same kernels in the same order as run_sweeps, so the same chain.
static int enqueue_sweeps(hsmc_ctx *ctx, int n_sweeps, bool npt) {
  if (n_sweeps <= 0) return HSMC_OK;
  if (ctx->small && ctx->cav_trace_cap == 0) {
    launch_sweep_small(ctx->sp, n_sweeps, npt, ctx->cavity, ctx->margin, ctx->small_smem, ctx->stream);
    ctx->sweep_base += (unsigned long long)n_sweeps;
    for (int l = 0; l < 2; l++)
      HSMC_CUDA(cudaMemsetAsync(ctx->sp.cnt[l], 0, sizeof(int) * (size_t)ctx->sp.ncell_alloc, ctx->stream));
    launch_build(ctx->sp, -1, ctx->num_sms, ctx->stream);
    reset_progress(ctx);
    return HSMC_OK;
  }
  int e = ensure_graph(ctx, npt);
  if (e) return e;
  const bool direct = ctx->cav_trace_cap > 0 || (ctx->flow && ctx->flow_graph == 0);
  int done = 0;
  if (!direct) {
    while (n_sweeps - done >= kGraphSweeps) {
      HSMC_CUDA(cudaGraphLaunch(npt ? ctx->graph_npt : ctx->graph, ctx->stream));
      done += kGraphSweeps;
    }
  }
  const int rest = n_sweeps - done;
  for (int s = 0; s < rest; s++) HSMC_CUDA(enqueue_sweep(ctx, s, false, npt));
  if (rest > 0) launch_advance(ctx->sp, rest, ctx->stream);
  ctx->sweep_base += (unsigned long long)n_sweeps;
  if (npt || ctx->cavity) rebuild_current_layout(ctx);
  return HSMC_OK;
}

static void drop_graphs(hsmc_ctx *ctx) {
  if (ctx->graph) cudaGraphExecDestroy(ctx->graph);
  if (ctx->graph_npt) cudaGraphExecDestroy(ctx->graph_npt);
  ctx->graph = ctx->graph_npt = nullptr;
}

// Lanes per cell and schedule; the grids follow.  Returns false when the
// combination cannot run on this device.
// flow: the schedule of hsmc_gpu_set_schedule (0, 1, 2 or 3).
static bool apply_schedule(hsmc_ctx *ctx, int flow, int group) {
  if (flow == 2) {  // one block: the lane mapping of the passes is kept for the other schedules
    if (ctx->small_smem == 0) return false;
    ctx->small = true;
    return true;
  }
  if (!move_pass_fits(group, ctx->sp.cap)) return false;
  ctx->small = false;
  int fg = 0;
  if (flow == 1) {
    int dev = 0, coop = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return false;
    fg = move_flow_grid(group, ctx->sp.cap, ctx->sp.ncell_alloc, ctx->num_sms);
    if (fg <= 0) return false;
  }
  ctx->group = group;
  ctx->flow = flow == 1;
  ctx->sp.olist = flow == 3 ? ctx->olist : nullptr;
  ctx->flow_grid = fg;
  ctx->pass_grid = move_pass_grid(group, ctx->sp.cap, ctx->sp.ncell_alloc, ctx->num_sms);
  ctx->flow_graph = -1;
  drop_graphs(ctx);
  return true;
}

// Every schedule and lane mapping that fits is timed on live sweeps: two
// rounds over the variants, each variant's timed run after an untimed one
// (its graph's first launch), and the fastest time of each variant kept, so
// that the system's drift during the tuning (from a lattice start, say)
// does not favour the variants timed last.
int hsmc_gpu_autotune(hsmc_ctx *ctx, int sweeps_per_variant, int *lanes_out) {
  if (!ctx || sweeps_per_variant <= 0 || !ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  const int options[4] = {1, 2, 4, 8};
  const bool was_profiling = ctx->profiling;
  const bool npt = ctx->prm.pressure > 0;
  const int sweeps = ((sweeps_per_variant + kGraphSweeps - 1) / kGraphSweeps) * kGraphSweeps;
  ctx->profiling = false;  // time the production path: graphs of sweeps
  const int g0 = ctx->group;
  double t[4][4];
  for (int f = 0; f < 4; f++)
    for (int v = 0; v < 4; v++) t[f][v] = 1e300;
  for (int round = 0; round < 2; round++)
    for (int f = 3; f >= 0; f--)
      for (int v = 0; v < 4; v++) {
        if (f == 2 && v > 0) continue;  // one variant
        if (!apply_schedule(ctx, f, f == 2 ? ctx->group : options[v])) continue;
        for (int rep = 0; rep < 2; rep++) {
          int e = run_sweeps(ctx, rep == 0 ? kGraphSweeps : sweeps, false, npt, nullptr);
          if (e) {
            ctx->profiling = was_profiling;
            return e;
          }
        }
        if (ctx->last_total_ms < t[f][v]) t[f][v] = ctx->last_total_ms;
      }
  int best_g = ctx->group, best_f = ctx->small ? 2 : (ctx->flow ? 1 : (ctx->sp.olist ? 3 : 0));
  double best_ms = 1e300;
  for (int f = 3; f >= 0; f--)
    for (int v = 0; v < 4; v++)
      if (t[f][v] < best_ms) {
        best_ms = t[f][v];
        best_f = f;
        best_g = f == 2 ? g0 : options[v];
      }
  ctx->profiling = was_profiling;
  if (best_f == 2) {
    apply_schedule(ctx, 0, g0);  // the lane mapping the other schedules fall back on
    ctx->small = true;
  } else {
    apply_schedule(ctx, best_f, best_g);
  }
  if (lanes_out) *lanes_out = best_g;
  return HSMC_OK;
}

// The reference's optimiser (opt_nvt / opt_npt / opt_cavity_nvt,
// src/optimizer.c:23-212) as one call: its opt_samples + 2 samples of
// opt_sweeps / opt_samples sweeps are enqueued back to back, each followed
// by k_opt_step, which sets the step for the next sample on the device; the
// host waits once, at the end.
int hsmc_gpu_optimize(hsmc_ctx *ctx, int opt_sweeps, int opt_samples, double part_target, double vol_target,
                      double out[4]) {
  if (!ctx || !ctx->uploaded || opt_samples <= 0 || opt_sweeps / opt_samples <= 0) return HSMC_ERR_INVALID_ARG;
  const bool npt = ctx->prm.pressure > 0;
  const int per = opt_sweeps / opt_samples;
  clear_counters_async(ctx);
  HSMC_CUDA(cudaMemsetAsync(&ctx->sp.st->status, 0, sizeof(int), ctx->stream));
  HSMC_CUDA(cudaMemsetAsync(&ctx->sp.st->opt_acc0, 0, 4 * sizeof(unsigned long long), ctx->stream));
  HSMC_CUDA(cudaEventRecord(ctx->ev_start, ctx->stream));
  for (int j = 0; j < opt_samples + 2; j++) {
    int e = enqueue_sweeps(ctx, per, npt);
    if (e) return e;
    launch_opt_step(ctx->sp, j, opt_samples, (unsigned long long)ctx->n * (unsigned long long)per * (j + 1),
                    part_target, vol_target, npt, ctx->stream);
  }
  HSMC_CUDA(cudaEventRecord(ctx->ev_stop, ctx->stream));
  int e = check_kernels(ctx);
  if (e) return e;
  timing_read(ctx);
  DevState s;
  if ((e = read_state(ctx, s))) return e;
  if (npt) HSMC_CUDA(cudaMemcpy(&ctx->hbox, ctx->sp.box, sizeof(Box), cudaMemcpyDeviceToHost));
  ctx->prm.dr_max = s.dr_max;
  ctx->prm.dv_max = s.dv_max;
  if (out) {
    out[0] = s.dr_max;
    out[1] = s.opt_a[1];
    out[2] = s.dv_max;
    out[3] = npt ? s.opt_av[1] : 0.0;
  }
  return s.status ? status_to_code(s.status) : HSMC_OK;
}

int hsmc_gpu_set_schedule(hsmc_ctx *ctx, int schedule, int lanes_per_cell) {
  if (!ctx || schedule < 0 || schedule > 3) return HSMC_ERR_INVALID_ARG;
  const int g = lanes_per_cell == 0 ? ctx->group : lanes_per_cell;
  if (g != 1 && g != 2 && g != 4 && g != 8) return HSMC_ERR_INVALID_ARG;
  return apply_schedule(ctx, schedule, g) ? HSMC_OK : HSMC_ERR_INVALID_ARG;
}

int hsmc_gpu_hold_region(hsmc_ctx *ctx, int region) {
  if (!ctx || region < -1 || region >= ctx->sp.ncell_alloc / 8) return HSMC_ERR_INVALID_ARG;
  HSMC_CUDA(cudaMemcpyAsync(&ctx->sp.st->flow_hold, &region, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  reset_progress(ctx);
  HSMC_CUDA(cudaStreamSynchronize(ctx->stream));
  return HSMC_OK;
}

int hsmc_gpu_get_schedule(hsmc_ctx *ctx, int *schedule, int *lanes_per_cell) {
  if (!ctx) return HSMC_ERR_INVALID_ARG;
  if (schedule) *schedule = ctx->small ? 2 : (ctx->flow ? 1 : (ctx->sp.olist ? 3 : 0));
  if (lanes_per_cell) *lanes_per_cell = ctx->group;
  return HSMC_OK;
}

int hsmc_gpu_sweeps(hsmc_ctx *ctx, int n_sweeps, uint64_t counters[6]) {
  if (!ctx || ctx->prm.pressure > 0) return HSMC_ERR_INVALID_ARG;
  return run_sweeps(ctx, n_sweeps, false, false, counters);
}

int hsmc_gpu_npt_sweeps(hsmc_ctx *ctx, int n_sweeps, uint64_t counters[6]) {
  if (!ctx || !(ctx->prm.pressure > 0)) return HSMC_ERR_INVALID_ARG;
  return run_sweeps(ctx, n_sweeps, false, true, counters);
}

int hsmc_gpu_sweeps_traced(hsmc_ctx *ctx, int n_sweeps, uint32_t *rec, int64_t capacity, int64_t *n_rec,
                           uint64_t counters[6]) {
  if (!ctx || !rec || capacity <= 0 || !n_rec) return HSMC_ERR_INVALID_ARG;
  HSMC_CUDA(ctx->trace.ensure(sizeof(uint32_t) * 12 * (size_t)capacity));
  ctx->sp.trace = (uint32_t *)ctx->trace.ptr;
  ctx->sp.trace_cap = (unsigned long long)capacity;
  int e = run_sweeps(ctx, n_sweeps, true, ctx->prm.pressure > 0, counters);
  ctx->sp.trace = nullptr;
  ctx->sp.trace_cap = 0;
  DevState s;
  int e2 = read_state(ctx, s);
  if (e2) return e2;
  const unsigned long long got = s.trace_count;
  *n_rec = (int64_t)got;
  if (got > (unsigned long long)capacity) return HSMC_ERR_INVALID_ARG;
  HSMC_CUDA(cudaMemcpy(rec, ctx->trace.ptr, sizeof(uint32_t) * 12 * got, cudaMemcpyDeviceToHost));
  return e;
}

int hsmc_gpu_get_box(hsmc_ctx *ctx, double out[5]) {
  if (!ctx || !out) return HSMC_ERR_INVALID_ARG;
  Box b;
  HSMC_CUDA(cudaMemcpyAsync(&b, ctx->sp.box, sizeof(Box), cudaMemcpyDeviceToHost, ctx->stream));
  HSMC_CUDA(cudaStreamSynchronize(ctx->stream));
  out[0] = b.len[0];
  out[1] = b.len[1];
  out[2] = b.len[2];
  out[3] = b.vol;
  out[4] = b.rho;
  return HSMC_OK;
}

int hsmc_gpu_grid_info(hsmc_ctx *ctx, int nc[3], float len32[3], float inv_w32[3], int *capacity) {
  if (!ctx) return HSMC_ERR_INVALID_ARG;
  for (int d = 0; d < 3; d++) {
    if (nc) nc[d] = ctx->hbox.nc[d];
    if (len32) len32[d] = ctx->hbox.len32[d];
    if (inv_w32) inv_w32[d] = ctx->hbox.inv_w32[d];
  }
  if (capacity) *capacity = ctx->sp.cap;
  return HSMC_OK;
}

// --------------------------------------------------- pair-count bins
// The bin of a pair at squared distance r2 is (int)((sqrt(r2) - 1) / dr)
// (rdf_hist_compute, src/compute_rdf.c:110-128; pressv_compute_hist,
// src/compute_press.c:123-165): correctly rounded operations, each
// monotone, so the bin is a step function of r2 and its steps fall at
// doubles that can be found once, by bisection over the bit patterns of
// positive doubles (which order as the doubles do).  The device then bins a
// pair by comparing r2 with them: the same bin for every double r2.
static double first_double_where(double lo, double hi, bool (*pred)(double, const double *), const double *arg) {
  uint64_t a, b;
  std::memcpy(&a, &lo, 8);
  std::memcpy(&b, &hi, 8);
  if (pred(lo, arg)) return lo;
  while (b - a > 1) {
    const uint64_t m = a + (b - a) / 2;
    double x;
    std::memcpy(&x, &m, 8);
    if (pred(x, arg)) b = m;
    else a = m;
  }
  double x;
  std::memcpy(&x, &b, 8);
  return x;
}

static bool bin_at_least(double r2, const double *a) { return (std::sqrt(r2) - 1.0) / a[0] >= a[1]; }
static bool root_at_least(double r2, const double *a) { return std::sqrt(r2) >= a[0]; }

extern "C" int hsmc_pair_thresholds(double dr, double rmax, int nbins, double *thr) {
  if (!thr || nbins <= 0 || !(dr > 0) || !(rmax > 1.0)) return HSMC_ERR_INVALID_ARG;
  const double hi = (rmax + dr + 1.0) * (rmax + dr + 1.0);  // above every threshold
  thr[0] = 1.0;
  for (int k = 1; k <= nbins; k++) {
    const double arg[2] = {dr, (double)k};
    thr[k] = first_double_where(1.0, hi, bin_at_least, arg);
  }
  const double arg[1] = {rmax};
  thr[nbins + 1] = first_double_where(1.0, hi, root_at_least, arg);
  return HSMC_OK;
}

static int pair_counts(hsmc_ctx *ctx, double dr, double rmax, int nbins, uint64_t *counts) {
  if (!ctx || !counts || nbins <= 0 || !(dr > 0) || !(rmax > 1.0) || !ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  HSMC_CUDA(ctx->hist.ensure(sizeof(unsigned long long) * (size_t)nbins));
  auto *d = (unsigned long long *)ctx->hist.ptr;
  HSMC_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long) * (size_t)nbins, ctx->stream));
  HSMC_CUDA(cudaMemsetAsync(&ctx->sp.st->status, 0, sizeof(int), ctx->stream));
  int k[3];
  stencil_for(ctx->hbox, rmax, k);
  // the bin thresholds, kept on the device while dr, rmax and nbins stay
  const double *thr = nullptr;
  if (nbins <= kFastBins) {
    if (ctx->thr_dr != dr || ctx->thr_rmax != rmax || ctx->thr_nbins != nbins) {
      ctx->thr_host.resize((size_t)nbins + 2);
      int e = hsmc_pair_thresholds(dr, rmax, nbins, ctx->thr_host.data());
      if (e) return e;
      HSMC_CUDA(ctx->thr.ensure(sizeof(double) * ctx->thr_host.size()));
      HSMC_CUDA(cudaMemcpy(ctx->thr.ptr, ctx->thr_host.data(), sizeof(double) * ctx->thr_host.size(),
                           cudaMemcpyHostToDevice));
      ctx->thr_dr = dr;
      ctx->thr_rmax = rmax;
      ctx->thr_nbins = nbins;
    }
    thr = (const double *)ctx->thr.ptr;
  }
  timing_begin(ctx);
  launch_pair_hist(ctx->sp, dr, rmax, nbins, d, k, ctx->stream, thr);
  timing_end(ctx);
  int e = check_kernels(ctx);
  if (e) return e;
  timing_read(ctx);
  HSMC_CUDA(cudaMemcpy(counts, d, sizeof(uint64_t) * (size_t)nbins, cudaMemcpyDeviceToHost));
  DevState s;
  if ((e = read_state(ctx, s))) return e;
  return s.status ? status_to_code(s.status) : HSMC_OK;
}

int hsmc_gpu_rdf(hsmc_ctx *ctx, double dr, double rmax, int nbins, uint64_t *counts) {
  return pair_counts(ctx, dr, rmax, nbins, counts);
}

int hsmc_gpu_pressv(hsmc_ctx *ctx, double dr, double rmax, int nbins, uint64_t *counts) {
  return pair_counts(ctx, dr, rmax, nbins, counts);
}

// --------------------------------------------------- allocation-free g(r)
// hsmc_gpu_rdf grows a device histogram with cudaMalloc whenever a caller
// asks for more bins than before.  Some callers cannot let a library
// allocate: a host program that hands all device memory to its own memory
// manager up front, or that runs under a fixed per-process memory budget on
// a GPU shared with other jobs, has nothing left to give; and a sampling loop
// with a hard time budget cannot absorb a first-call cudaMalloc, which may
// synchronise the device.  For them the counts go into the fixed array
// below, compiled into the library and resident on every GPU that loads it
// until the process exits.  In host code the symbol is only a stand-in for
// the device array: its device address is looked up once per device with
// cudaGetSymbolAddress and that address is what the kernel receives.
// Every call shares this array and clears it before counting, so two calls
// that run at the same time on one GPU (different contexts or streams)
// race on it.
static __device__ __align__(256) unsigned long long g_rdf_noalloc_bins[HSMC_RDF_NOALLOC_MAX_BINS];

// The address is looked up once per device.  Several contexts may be driven
// from different host threads, so the first calls on a device can meet here:
// the lookup runs under a mutex and the address is published with a release
// store, which the unlocked fast path reads with an acquire load (a thread
// never sees a non-null entry before the address it holds).
static std::mutex g_noalloc_mu;
static std::atomic<unsigned long long *> g_noalloc_addr[256];

static unsigned long long *noalloc_bins_on(int device, int *status) {
  *status = HSMC_OK;
  if (device < 0 || device >= 256) {
    *status = HSMC_ERR_NO_DEVICE;
    return nullptr;
  }
  unsigned long long *a = g_noalloc_addr[device].load(std::memory_order_acquire);
  if (a) return a;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  a = g_noalloc_addr[device].load(std::memory_order_relaxed);
  if (!a) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_rdf_noalloc_bins);
    if (e != cudaSuccess || p == nullptr) {
      *status = cuda_status(e != cudaSuccess ? e : cudaErrorInvalidSymbol);
      return nullptr;
    }
    a = static_cast<unsigned long long *>(p);
    g_noalloc_addr[device].store(a, std::memory_order_release);
  }
  return a;
}

int hsmc_gpu_rdf_noalloc(hsmc_ctx *ctx, double dr, double rmax, int nbins, uint64_t *counts) {
  if (!ctx || !counts || nbins <= 0 || !(dr > 0) || !(rmax > 1.0) || !ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  if (nbins > HSMC_RDF_NOALLOC_MAX_BINS) {
    fprintf(stderr, "hsmc_gpu_rdf_noalloc: %d bins requested, at most %d are available\n", nbins,
            HSMC_RDF_NOALLOC_MAX_BINS);
    return HSMC_ERR_INVALID_ARG;
  }
  // The array's address is looked up with the context's device current.
  cudaPointerAttributes attr{};
  HSMC_CUDA(cudaPointerGetAttributes(&attr, ctx->sp.pos));
  int current = 0;
  HSMC_CUDA(cudaGetDevice(&current));
  if (current != attr.device) HSMC_CUDA(cudaSetDevice(attr.device));
  int st = HSMC_OK;
  unsigned long long *d = noalloc_bins_on(attr.device, &st);
  int e = st;
  if (!e) {
    cudaError_t ce = cudaMemsetAsync(d, 0, sizeof(unsigned long long) * (size_t)nbins, ctx->stream);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(&ctx->sp.st->status, 0, sizeof(int), ctx->stream);
    if (ce != cudaSuccess) e = cuda_status(ce);
  }
  if (!e) {
    int k[3];
    stencil_for(ctx->hbox, rmax, k);
    launch_pair_hist(ctx->sp, dr, rmax, nbins, d, k, ctx->stream);
    e = check_kernels(ctx);
  }
  if (!e) {
    cudaError_t ce = cudaMemcpyAsync(counts, d, sizeof(uint64_t) * (size_t)nbins, cudaMemcpyDeviceToHost, ctx->stream);
    if (ce != cudaSuccess) e = cuda_status(ce);
  }
  DevState s;
  if (!e) e = read_state(ctx, s);
  if (!e && s.status) e = status_to_code(s.status);
  if (current != attr.device) cudaSetDevice(current);
  return e;
}

static int scaled_scan(hsmc_ctx *ctx, const double *sf, int n_sf, unsigned long long mask[4]) {
  if (!ctx || !sf || n_sf <= 0 || n_sf > 256 || !ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  double smallest = 1.0;
  for (int k = 0; k < n_sf; k++) {
    if (!(sf[k] > 0.5 && sf[k] <= 1.0)) return HSMC_ERR_INVALID_ARG;
    smallest = sf[k] < smallest ? sf[k] : smallest;
  }
  clear_counters_async(ctx);
  int k[3];
  stencil_for(ctx->hbox, 1.0 / smallest, k);
  timing_begin(ctx);
  launch_scaled_scan(ctx->sp, sf, n_sf, k, ctx->stream);
  timing_end(ctx);
  int e = check_kernels(ctx);
  if (e) return e;
  timing_read(ctx);
  DevState s;
  if ((e = read_state(ctx, s))) return e;
  for (int w = 0; w < 4; w++) mask[w] = s.scan_mask[w];
  return HSMC_OK;
}

int hsmc_gpu_presst(hsmc_ctx *ctx, const double *sf, int n_sf, uint64_t *nonoverlap) {
  if (!nonoverlap) return HSMC_ERR_INVALID_ARG;
  unsigned long long m[4];
  int e = scaled_scan(ctx, sf, n_sf, m);
  if (e) return e;
  for (int k = 0; k < n_sf; k++) nonoverlap[k] = ((m[k >> 6] >> (k & 63)) & 1ull) ? 0 : 1;
  return HSMC_OK;
}

int hsmc_gpu_scan_overlap(hsmc_ctx *ctx, double sf, int *overlap) {
  if (!ctx || !overlap || !ctx->uploaded || !(sf > 0.5 && sf <= 2.0)) return HSMC_ERR_INVALID_ARG;
  // The kernel the NpT volume move runs, on a caller-given scale factor.
  const int zero = 0;
  HSMC_CUDA(cudaMemcpyAsync(&ctx->sp.st->vol_sf, &sf, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  HSMC_CUDA(cudaMemcpyAsync(&ctx->sp.st->vol_overlap, &zero, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  timing_begin(ctx);
  launch_volume_scan(ctx->sp, ctx->stream);
  timing_end(ctx);
  int e = check_kernels(ctx);
  if (e) return e;
  timing_read(ctx);
  int ov = 0;
  HSMC_CUDA(cudaMemcpy(&ov, &ctx->sp.st->vol_overlap, sizeof(int), cudaMemcpyDeviceToHost));
  *overlap = ov ? 1 : 0;
  return HSMC_OK;
}

int hsmc_gpu_widom(hsmc_ctx *ctx, int64_t n_insertions, uint64_t *accepted) {
  if (!ctx || !accepted || n_insertions < 0 || !ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  clear_counters_async(ctx);
  timing_begin(ctx);
  launch_widom(ctx->sp, n_insertions, ctx->widom_seq, nullptr, nullptr, ctx->stream);
  timing_end(ctx);
  int e = check_kernels(ctx);
  if (e) return e;
  timing_read(ctx);
  ctx->widom_seq++;
  DevState s;
  if ((e = read_state(ctx, s))) return e;
  *accepted = s.widom_ok;
  return HSMC_OK;
}

int hsmc_gpu_widom_replay(hsmc_ctx *ctx, const double *pos, int n, uint8_t *overlap) {
  if (!ctx || !pos || !overlap || n < 0 || !ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  if (n == 0) return HSMC_OK;
  HSMC_CUDA(ctx->qpos.ensure(sizeof(double) * 3 * (size_t)n));
  HSMC_CUDA(ctx->flags.ensure((size_t)n));
  HSMC_CUDA(cudaMemcpyAsync(ctx->qpos.ptr, pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  clear_counters_async(ctx);
  launch_widom(ctx->sp, n, 0, (const double *)ctx->qpos.ptr, (uint8_t *)ctx->flags.ptr, ctx->stream);
  int e = check_kernels(ctx);
  if (e) return e;
  HSMC_CUDA(cudaMemcpy(overlap, ctx->flags.ptr, (size_t)n, cudaMemcpyDeviceToHost));
  return HSMC_OK;
}

int hsmc_gpu_overlap_replay(hsmc_ctx *ctx, const int *ids, const double *pos, int n, uint8_t *overlap) {
  if (!ctx || !ids || !pos || !overlap || n < 0 || !ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  if (n == 0) return HSMC_OK;
  for (int k = 0; k < n; k++)
    if (ids[k] < 0 || ids[k] >= ctx->n) return HSMC_ERR_INVALID_ARG;
  HSMC_CUDA(ctx->qpos.ensure(sizeof(double) * 3 * (size_t)n));
  HSMC_CUDA(ctx->qids.ensure(sizeof(int) * (size_t)n));
  HSMC_CUDA(ctx->flags.ensure((size_t)n));
  HSMC_CUDA(cudaMemcpyAsync(ctx->qpos.ptr, pos, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  HSMC_CUDA(cudaMemcpyAsync(ctx->qids.ptr, ids, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  launch_overlap_replay(ctx->sp, (const int *)ctx->qids.ptr, (const double *)ctx->qpos.ptr, n,
                        (uint8_t *)ctx->flags.ptr, ctx->stream);
  int e = check_kernels(ctx);
  if (e) return e;
  HSMC_CUDA(cudaMemcpy(overlap, ctx->flags.ptr, (size_t)n, cudaMemcpyDeviceToHost));
  return HSMC_OK;
}

int hsmc_gpu_ql(hsmc_ctx *ctx, int l, double rc, double *ql_mean, double *per_particle) {
  if (!ctx || !ql_mean || l < 0 || l > 12 || !(rc > 0) || !ctx->uploaded) return HSMC_ERR_INVALID_ARG;
  HSMC_CUDA(ctx->qbuf.ensure(sizeof(double) * ((size_t)ctx->n + 1)));
  double *q = (double *)ctx->qbuf.ptr;
  int k[3];
  stencil_for(ctx->hbox, rc, k);
  timing_begin(ctx);
  launch_ql(ctx->sp, l, rc, k, q, q + ctx->n, ctx->stream);
  timing_end(ctx);
  int e = check_kernels(ctx);
  if (e) return e;
  timing_read(ctx);
  double sum = 0.0;
  HSMC_CUDA(cudaMemcpy(&sum, q + ctx->n, sizeof(double), cudaMemcpyDeviceToHost));
  if (per_particle) HSMC_CUDA(cudaMemcpy(per_particle, q, sizeof(double) * (size_t)ctx->n, cudaMemcpyDeviceToHost));
  *ql_mean = sum / ctx->n;
  return HSMC_OK;
}

// Geometric cluster moves (cluster.cu): one cooperative launch makes the
// moves one after the other and rebuilds the current layout after each.
static int cluster_run(hsmc_ctx *ctx, int n_moves, const double *pivot, int axis, int seed_particle,
                       int64_t *sizes, double *drawn) {
  if (!ctx || n_moves < 0 || !ctx->uploaded || ctx->prm.pressure > 0) return HSMC_ERR_INVALID_ARG;
  if (n_moves == 0) return HSMC_OK;
  const size_t n = (size_t)ctx->n;
  if (!ctx->cl_mark.ptr) {
    HSMC_CUDA(ctx->cl_mark.ensure(sizeof(uint32_t) * n));
    HSMC_CUDA(cudaMemsetAsync(ctx->cl_mark.ptr, 0, sizeof(uint32_t) * n, ctx->stream));
    ctx->cl_epoch = 0;
  }
  HSMC_CUDA(ctx->cl_queue.ensure(sizeof(int) * n));
  HSMC_CUDA(ctx->cl_ctr.ensure(sizeof(uint32_t) * 4));
  const size_t per = sizeof(long long) + 5 * sizeof(double);
  HSMC_CUDA(ctx->cl_out.ensure(per * (size_t)n_moves));
  if (ctx->cl_grid < 0) ctx->cl_grid = cluster_grid(ctx->n, ctx->hbox.ncell, ctx->num_sms);
  long long *d_size = (long long *)ctx->cl_out.ptr;
  double *d_drawn = (double *)(d_size + n_moves);
  HSMC_CUDA(cudaMemsetAsync(&ctx->sp.st->status, 0, sizeof(int), ctx->stream));
  ClusterJob job{};
  job.queue = (int *)ctx->cl_queue.ptr;
  job.mark = (uint32_t *)ctx->cl_mark.ptr;
  job.ctr = (uint32_t *)ctx->cl_ctr.ptr;
  job.sint = std::sin(M_PI);
  if (std::cos(M_PI) != -1.0) return HSMC_ERR_INVALID_ARG;  // the folded rotation assumes it
  if (pivot) {
    job.given = 1;
    for (int d = 0; d < 3; d++) job.pivot[d] = pivot[d];
    job.axis = axis;
    job.seed_id = seed_particle;
  }
  // epochs cl_epoch + 1 .. cl_epoch + n_moves; marks are cleared before the
  // counter could come round to an epoch an old mark still holds
  if ((unsigned long long)ctx->cl_epoch + (unsigned long long)n_moves > 0xFFFFFFFFull) {
    HSMC_CUDA(cudaMemsetAsync(ctx->cl_mark.ptr, 0, sizeof(uint32_t) * n, ctx->stream));
    ctx->cl_epoch = 0;
  }
  job.epoch = ctx->cl_epoch + 1u;
  job.seq = ctx->cluster_seq;
  job.size_out = d_size;
  job.drawn = d_drawn;
  HSMC_CUDA(cudaMemsetAsync(job.ctr, 0, sizeof(uint32_t) * 4, ctx->stream));
  HSMC_CUDA(launch_cluster(ctx->sp, job, n_moves, ctx->cl_grid, ctx->hbox.ncell, ctx->stream));
  if (ctx->cl_grid == 0) rebuild_current_layout(ctx);  // the one-block kernel moved only the positions
  else ctx->cl_epoch += (uint32_t)n_moves;
  if (!pivot) ctx->cluster_seq += (unsigned long long)n_moves;
  int e = check_kernels(ctx);
  if (e) return e;
  DevState s;
  if ((e = read_state(ctx, s))) return e;
  if (s.status) return status_to_code(s.status);
  if (sizes) {
    std::vector<long long> h((size_t)n_moves);
    HSMC_CUDA(cudaMemcpy(h.data(), d_size, sizeof(long long) * (size_t)n_moves, cudaMemcpyDeviceToHost));
    for (int k = 0; k < n_moves; k++) sizes[k] = (int64_t)h[(size_t)k];
  }
  if (drawn) HSMC_CUDA(cudaMemcpy(drawn, d_drawn, sizeof(double) * 5 * (size_t)n_moves, cudaMemcpyDeviceToHost));
  return HSMC_OK;
}

int hsmc_gpu_cavity_psi(hsmc_ctx *ctx, const double *x, int n, double *out) {
  if (!ctx || n < 0 || (n > 0 && (!x || !out)) || !ctx->cavity) return HSMC_ERR_INVALID_ARG;
  if (n == 0) return HSMC_OK;
  HSMC_CUDA(ctx->qpos.ensure(sizeof(double) * 2 * (size_t)n));
  double *d = (double *)ctx->qpos.ptr;
  HSMC_CUDA(cudaMemcpyAsync(d, x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
  launch_cavity_psi(ctx->sp, d, n, d + n, ctx->stream);
  HSMC_CUDA(cudaMemcpyAsync(out, d + n, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
  return check_kernels(ctx);
}

int hsmc_gpu_cavity_trace(hsmc_ctx *ctx, int64_t capacity) {
  if (!ctx || capacity < 0 || !ctx->cavity) return HSMC_ERR_INVALID_ARG;
  if (capacity > 0) HSMC_CUDA(ctx->cav_trace.ensure(32 * (size_t)capacity));
  ctx->cav_trace_cap = capacity;
  HSMC_CUDA(cudaMemsetAsync(&ctx->sp.st->cav_trace_count, 0, sizeof(unsigned long long), ctx->stream));
  return check_kernels(ctx);
}

int hsmc_gpu_cavity_trace_read(hsmc_ctx *ctx, uint32_t *rec, int64_t capacity, int64_t *n_rec) {
  if (!ctx || !n_rec || capacity < 0 || (capacity > 0 && !rec) || !ctx->cavity) return HSMC_ERR_INVALID_ARG;
  unsigned long long count = 0;
  HSMC_CUDA(cudaMemcpy(&count, &ctx->sp.st->cav_trace_count, sizeof(count), cudaMemcpyDeviceToHost));
  long long k = (long long)count;
  if (k > ctx->cav_trace_cap) k = ctx->cav_trace_cap;
  if (k > capacity) k = capacity;
  if (k > 0) HSMC_CUDA(cudaMemcpy(rec, ctx->cav_trace.ptr, 32 * (size_t)k, cudaMemcpyDeviceToHost));
  *n_rec = k;
  HSMC_CUDA(cudaMemsetAsync(&ctx->sp.st->cav_trace_count, 0, sizeof(unsigned long long), ctx->stream));
  return check_kernels(ctx);
}

int hsmc_gpu_cluster_moves(hsmc_ctx *ctx, int n_moves, int64_t *sizes, double *drawn) {
  return cluster_run(ctx, n_moves, nullptr, 0, 0, sizes, drawn);
}

int hsmc_gpu_cluster_move_at(hsmc_ctx *ctx, const double pivot[3], int axis, int seed_particle, int64_t *size) {
  if (!ctx || !pivot || axis < 0 || axis > 2 || seed_particle < 0 || seed_particle >= ctx->n)
    return HSMC_ERR_INVALID_ARG;
  for (int d = 0; d < 3; d++)
    if (!(pivot[d] >= 0.0 && pivot[d] <= ctx->hbox.len[d])) return HSMC_ERR_INVALID_ARG;
  return cluster_run(ctx, 1, pivot, axis, seed_particle, size, nullptr);
}

int hsmc_gpu_rng_state(hsmc_ctx *ctx, uint64_t out[4]) {
  if (!ctx || !out) return HSMC_ERR_INVALID_ARG;
  out[0] = ctx->prm.seed;
  out[1] = ctx->sweep_base;
  out[2] = ctx->widom_seq;
  out[3] = ctx->cluster_seq;
  return HSMC_OK;
}

int hsmc_gpu_rng_set_state(hsmc_ctx *ctx, const uint64_t st[4]) {
  if (!ctx || !st || st[1] == 0) return HSMC_ERR_INVALID_ARG;
  ctx->prm.seed = st[0];
  ctx->sweep_base = st[1];
  ctx->widom_seq = st[2];
  ctx->cluster_seq = st[3];
  HSMC_CUDA(cudaMemcpyAsync(&ctx->sp.st->seed, &st[0], sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream));
  HSMC_CUDA(cudaMemcpyAsync(&ctx->sp.st->sweep_base, &st[1], sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream));
  reset_progress(ctx);
  if (ctx->uploaded) {
    // The layout a sweep writes follows the parity of its index: rebuild the
    // current one for the new position in the stream.
    SysPtrs &sp = ctx->sp;
    for (int l = 0; l < 2; l++)
      HSMC_CUDA(cudaMemsetAsync(sp.cnt[l], 0, sizeof(int) * (size_t)sp.ncell_alloc, ctx->stream));
    launch_build(sp, -1, ctx->num_sms, ctx->stream);
    int e = check_kernels(ctx);
    if (e) return e;
  }
  HSMC_CUDA(cudaStreamSynchronize(ctx->stream));
  return HSMC_OK;
}

}  // extern "C"
