// Batched replicas (include/hsmc_gpu.h, hsmc_batch_*): many independent NVT
// systems of different size and density advanced together.  All replicas
// live in pooled device buffers; a device table holds one SysPtrs per
// replica, and every kernel of a sweep covers all of them in one launch
// (blockIdx.y = replica).  Sweeps run as CUDA graphs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <vector>

#include "../../include/hsmc_gpu.h"
#include "engine.cuh"

using namespace hsmc;

namespace hsmc {
// batch_persist.cu
int batch_persist_max_reps();
int batch_persist_max_clusters(int cap, int cluster_blocks);
cudaError_t prepare_batch_persist();
cudaError_t launch_batch_persist(int cap, const SysPtrs *reps, const int *rep_ids, const int *nstart,
                                 const int *gstart, const int *cstart, const int *bundle, int n_bundles,
                                 int n_sweeps, int cluster_blocks, cudaStream_t s);
int batch_grid_blocks(int cap, int num_sms);
cudaError_t prepare_batch_grid();
cudaError_t launch_batch_grid(int cap, const SysPtrs *reps, const int *rep_ids, const int *nstart, const int *gstart,
                              const int *cstart, void *params, unsigned *bar, int *abort, unsigned *work,
                              int *status, int n_reps, int n_sweeps, int blocks, cudaStream_t s);
}  // namespace hsmc

namespace {

constexpr int kBatchGraphSweeps = 8;

int cuda_fail(cudaError_t e) {
  fprintf(stderr, "hsmc_gpu: CUDA error %s\n", cudaGetErrorString(e));
  return HSMC_ERR_CUDA;
}

#define BATCH_CUDA(call)                    \
  do {                                      \
    cudaError_t e_ = (call);                \
    if (e_ != cudaSuccess) return cuda_fail(e_); \
  } while (0)

int code_of(int st) {
  if (st & ST_FLOW_TIMEOUT) return HSMC_ERR_TIMEOUT;
  if (st & (ST_CELL_OVERFLOW | ST_BAD_CELL)) return HSMC_ERR_CELL_OVERFLOW;
  if (st & ST_BAD_BIN) return HSMC_ERR_BAD_BIN;
  if (st & ST_OUT_OF_BOX) return HSMC_ERR_OUT_OF_BOX;
  return HSMC_OK;
}

}  // namespace

struct hsmc_batch {
  int reps = 0;
  // replicas of one cell capacity move in one flat launch; lanes per cell
  // grow with the capacity so a block's shared memory stays the same
  struct CapClass {
    int cap = 8, group = 2, n = 0, tot_groups = 0;
    SysPtrs *d_reps = nullptr;
    int *d_gstart = nullptr, *d_ids = nullptr;
    // schedule 3: prefix sums of the replicas' cells, the occupancy counts
    // and one list per pass of (replica, cell) pairs
    long long n_cells = 0;
    int *d_cstart = nullptr, *d_ocnt = nullptr, *d_olist = nullptr;
  };
  std::vector<CapClass> classes;
  int max_n = 0, max_ncell = 0;
  int tot_n = 0, tot_groups = 0;   // particles and active cells (one colour) of all replicas
  long long tot_cell = 0;
  int *d_nstart = nullptr, *d_gstart = nullptr;  // their prefix sums by replica (n_reps + 1)
  cudaStream_t stream = nullptr;
  std::vector<hsmc_params> prm;
  std::vector<SysPtrs> sp;  // host copies of the device table
  std::vector<Box> hbox;
  std::vector<char> uploaded;
  SysPtrs *d_reps = nullptr;
  double *pos = nullptr;
  int *cnt[2] = {nullptr, nullptr};
  Slot *slot[2] = {nullptr, nullptr};
  Box *box = nullptr;
  DevState *st = nullptr;
  unsigned long long *hist = nullptr;
  size_t hist_bins = 0;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.0;
  // schedule 1: every sweep of a call in one launch of thread-block
  // clusters, one cluster per bundle of replicas (batch_persist.cu);
  // schedule 3: the flat launches with every pass's cells in occupancy order
  int schedule = 0;
  int cluster_blocks = 4, tile = 2;
  struct Bundles {
    int cap = 8, n_bundles = 0;
    SysPtrs *d_reps = nullptr;
    int *d_ids = nullptr, *d_nstart = nullptr, *d_gstart = nullptr, *d_cstart = nullptr, *d_bundle = nullptr;
  };
  std::vector<Bundles> bundles;  // per cell capacity, for (bundled_cb, bundled_tile)
  int bundled_cb = 0, bundled_tile = 0;
  int persist_graph_sweeps = 0;
  cudaGraphExec_t persist_graph = nullptr;  // one persistent launch per class, for persist_graph_sweeps
  // schedule 2: every sweep of a call in one cooperative launch per cell
  // capacity over the whole device (batch_persist.cu, k_batch_grid)
  struct GridClass {
    int cap = 8, n = 0, blocks = 0;
    SysPtrs *d_reps = nullptr;
    int *d_ids = nullptr, *d_nstart = nullptr, *d_gstart = nullptr, *d_cstart = nullptr;
    void *d_params = nullptr;
    unsigned *d_bar = nullptr;  // barrier words, the abort flag and two work counters
    int *status = nullptr;      // the class's first replica's status
  };
  std::vector<GridClass> grids;
};

static void free_grids(hsmc_batch *b) {
  for (auto &q : b->grids) {
    cudaFree(q.d_reps);
    cudaFree(q.d_ids);
    cudaFree(q.d_nstart);
    cudaFree(q.d_gstart);
    cudaFree(q.d_cstart);
    cudaFree(q.d_params);
    cudaFree(q.d_bar);
  }
  b->grids.clear();
}

static void free_bundles(hsmc_batch *b) {
  for (auto &q : b->bundles) {
    cudaFree(q.d_reps);
    cudaFree(q.d_ids);
    cudaFree(q.d_nstart);
    cudaFree(q.d_gstart);
    cudaFree(q.d_cstart);
    cudaFree(q.d_bundle);
  }
  b->bundles.clear();
  b->bundled_cb = b->bundled_tile = 0;
  if (b->persist_graph) cudaGraphExecDestroy(b->persist_graph);
  b->persist_graph = nullptr;
  b->persist_graph_sweeps = 0;
}

static int batch_check(hsmc_batch *b) {
  BATCH_CUDA(cudaGetLastError());
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  return HSMC_OK;
}

static int batch_status(hsmc_batch *b, std::vector<DevState> &out) {
  out.resize(b->reps);
  BATCH_CUDA(cudaMemcpyAsync(out.data(), b->st, sizeof(DevState) * b->reps, cudaMemcpyDeviceToHost, b->stream));
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  for (const DevState &s : out)
    if (s.status) return code_of(s.status);
  return HSMC_OK;
}

extern "C" {

void hsmc_batch_destroy(hsmc_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  free_bundles(b);
  free_grids(b);
  cudaFree(b->d_reps);
  cudaFree(b->d_nstart);
  cudaFree(b->d_gstart);
  for (auto &q : b->classes) {
    cudaFree(q.d_reps);
    cudaFree(q.d_ids);
    cudaFree(q.d_gstart);
    cudaFree(q.d_cstart);
    cudaFree(q.d_ocnt);
    cudaFree(q.d_olist);
  }
  cudaFree(b->pos);
  for (int l = 0; l < 2; l++) {
    cudaFree(b->cnt[l]);
    cudaFree(b->slot[l]);
  }
  cudaFree(b->box);
  cudaFree(b->st);
  cudaFree(b->hist);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

int hsmc_batch_create(const hsmc_params *params, int n_systems, hsmc_batch **out) {
  if (!params || !out || n_systems <= 0 || n_systems > 65535) return HSMC_ERR_INVALID_ARG;
  *out = nullptr;
  int dev = 0;
  cudaDeviceProp dp{};
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&dp, dev) != cudaSuccess)
    return HSMC_ERR_NO_DEVICE;
  if (!(dp.major == 10 && dp.minor == 3)) return HSMC_ERR_NO_DEVICE;
  hsmc_batch *b = new hsmc_batch();
  b->reps = n_systems;
  b->prm.assign(params, params + n_systems);
  b->hbox.resize(n_systems);
  b->sp.resize(n_systems);
  b->uploaded.assign(n_systems, 0);
  size_t tot_n = 0, tot_cell = 0;
  std::vector<int> caps(n_systems, 8);
  size_t tot_slot = 0;
  for (int k = 0; k < n_systems; k++) {
    const hsmc_params &p = params[k];
    if (p.n_particles <= 0 || p.pressure > 0 || !(p.dr_max >= 0)) {
      delete b;
      return HSMC_ERR_INVALID_ARG;
    }
    for (int d = 0; d < 3; d++)
      if (!(p.box[d] > 0) || !(p.dr_max < p.box[d])) {
        delete b;
        return HSMC_ERR_INVALID_ARG;
      }
    int ck = 8;
    const double rho = p.rho > 0 ? p.rho : p.n_particles / (p.box[0] * p.box[1] * p.box[2]);
    if (!(p.min_cell_edge >= 0.0)) {
      delete b;
      return HSMC_ERR_INVALID_ARG;
    }
    int e = make_box(p.box, rho, b->hbox[k], ck, p.min_cell_edge);
    if (e) {
      delete b;
      return e;
    }
    caps[k] = ck;
    tot_slot += (size_t)b->hbox[k].ncell * ck;
    tot_n += (size_t)p.n_particles;
    tot_cell += (size_t)b->hbox[k].ncell;
    b->max_n = p.n_particles > b->max_n ? p.n_particles : b->max_n;
    b->max_ncell = b->hbox[k].ncell > b->max_ncell ? b->hbox[k].ncell : b->max_ncell;
  }
  auto fail = [&](cudaError_t e) {
    hsmc_batch_destroy(b);
    return cuda_fail(e);
  };
  cudaError_t ce;
  prepare_move_pass();
  if ((ce = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking)) != cudaSuccess) return fail(ce);
  if ((ce = cudaMalloc(&b->pos, sizeof(double) * 4 * tot_n)) != cudaSuccess) return fail(ce);
  for (int l = 0; l < 2; l++) {
    if ((ce = cudaMalloc(&b->cnt[l], sizeof(int) * tot_cell)) != cudaSuccess) return fail(ce);
    if ((ce = cudaMemset(b->cnt[l], 0, sizeof(int) * tot_cell)) != cudaSuccess) return fail(ce);
    if ((ce = cudaMalloc(&b->slot[l], sizeof(Slot) * tot_slot)) != cudaSuccess) return fail(ce);
  }
  if ((ce = cudaMalloc(&b->box, sizeof(Box) * n_systems)) != cudaSuccess) return fail(ce);
  if ((ce = cudaMalloc(&b->st, sizeof(DevState) * n_systems)) != cudaSuccess) return fail(ce);
  if ((ce = cudaMalloc(&b->d_reps, sizeof(SysPtrs) * n_systems)) != cudaSuccess) return fail(ce);
  std::vector<DevState> st0(n_systems);
  size_t on = 0, oc = 0, os = 0;
  for (int k = 0; k < n_systems; k++) {
    SysPtrs &s = b->sp[k];
    s.pos = b->pos + 4 * on;
    for (int l = 0; l < 2; l++) {
      s.cnt[l] = b->cnt[l] + oc;
      s.slot[l] = b->slot[l] + os;
    }
    s.box = b->box + k;
    s.st = b->st + k;
    s.trace = nullptr;
    s.trace_cap = 0;
    s.n = params[k].n_particles;
    s.cap = caps[k];
    s.ncell_alloc = b->hbox[k].ncell;
    DevState &d = st0[k];
    d = DevState{};
    d.sweep_base = 1;
    d.dr_max = params[k].dr_max;
    d.dv_max = params[k].dv_max;
    d.seed = params[k].seed;
    d.per_cell = params[k].lattice_type == 1 ? 1 : 4;
    d.flow_hold = -1;
    for (int q = 0; q < 3; q++) {
      d.cells[q] = params[k].cells[q];
      d.nc_alloc[q] = b->hbox[k].nc[q];
    }
    on += (size_t)params[k].n_particles;
    oc += (size_t)b->hbox[k].ncell;
    os += (size_t)b->hbox[k].ncell * caps[k];
  }
  if ((ce = cudaMemcpy(b->box, b->hbox.data(), sizeof(Box) * n_systems, cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(ce);
  if ((ce = cudaMemcpy(b->st, st0.data(), sizeof(DevState) * n_systems, cudaMemcpyHostToDevice)) != cudaSuccess)
    return fail(ce);
  if ((ce = cudaMemcpy(b->d_reps, b->sp.data(), sizeof(SysPtrs) * n_systems, cudaMemcpyHostToDevice)) !=
      cudaSuccess)
    return fail(ce);
  // flat launches: prefix sums of particles and of active cells per replica
  {
    std::vector<int> ns(n_systems + 1, 0), gs(n_systems + 1, 0);
    long long tn = 0, tg = 0;
    for (int k = 0; k < n_systems; k++) {
      ns[k] = (int)tn;
      gs[k] = (int)tg;
      tn += params[k].n_particles;
      tg += (long long)b->hbox[k].ncell / 8;
    }
    if (tn > 0x7fffffffll || tg * 8 > 0x7fffffffll) return fail(cudaErrorInvalidValue);
    ns[n_systems] = (int)tn;
    gs[n_systems] = (int)tg;
    b->tot_n = (int)tn;
    b->tot_groups = (int)tg;
    b->tot_cell = (long long)oc;
    if ((ce = cudaMalloc(&b->d_nstart, sizeof(int) * (n_systems + 1))) != cudaSuccess) return fail(ce);
    if ((ce = cudaMalloc(&b->d_gstart, sizeof(int) * (n_systems + 1))) != cudaSuccess) return fail(ce);
    if ((ce = cudaMemcpy(b->d_nstart, ns.data(), sizeof(int) * (n_systems + 1), cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(b->d_gstart, gs.data(), sizeof(int) * (n_systems + 1), cudaMemcpyHostToDevice)))
      return fail(ce);
  }
  for (int c : {8, 16, 32}) {
    std::vector<SysPtrs> sp;
    std::vector<int> ids, gs(1, 0), cs(1, 0);
    for (int k = 0; k < n_systems; k++)
      if (caps[k] == c) {
        sp.push_back(b->sp[k]);
        ids.push_back(k);
        gs.push_back(gs.back() + b->hbox[k].ncell / 8);
        cs.push_back(cs.back() + b->hbox[k].ncell);
      }
    if (sp.empty()) continue;
    hsmc_batch::CapClass cl;
    cl.cap = c;
    cl.group = c / 4;
    cl.n = (int)sp.size();
    cl.tot_groups = gs.back();
    cl.n_cells = cs.back();
    b->classes.push_back(cl);
    hsmc_batch::CapClass &q = b->classes.back();
    if ((ce = cudaMalloc(&q.d_reps, sizeof(SysPtrs) * q.n)) || (ce = cudaMalloc(&q.d_ids, sizeof(int) * q.n)) ||
        (ce = cudaMalloc(&q.d_gstart, sizeof(int) * (q.n + 1))) ||
        (ce = cudaMalloc(&q.d_cstart, sizeof(int) * (q.n + 1))) ||
        (ce = cudaMalloc(&q.d_ocnt, sizeof(int) * (size_t)kOrderWords)) ||
        (ce = cudaMalloc(&q.d_olist, sizeof(int) * 2 * 8 * (size_t)q.tot_groups)))
      return fail(ce);
    if ((ce = cudaMemcpy(q.d_reps, sp.data(), sizeof(SysPtrs) * q.n, cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_ids, ids.data(), sizeof(int) * q.n, cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_gstart, gs.data(), sizeof(int) * (q.n + 1), cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_cstart, cs.data(), sizeof(int) * (q.n + 1), cudaMemcpyHostToDevice)) ||
        (ce = cudaMemset(q.d_ocnt, 0, sizeof(int) * (size_t)kOrderWords)))
      return fail(ce);
  }
  if ((ce = cudaEventCreate(&b->ev0)) != cudaSuccess) return fail(ce);
  if ((ce = cudaEventCreate(&b->ev1)) != cudaSuccess) return fail(ce);
  *out = b;
  return HSMC_OK;
}

int hsmc_batch_upload_config(hsmc_batch *b, int k, const double (*conf)[4], int n) {
  if (!b || k < 0 || k >= b->reps || !conf || n != b->sp[k].n) return HSMC_ERR_INVALID_ARG;
  const Box &bx = b->hbox[k];
  for (int i = 0; i < n; i++) {
    if (conf[i][0] != (double)i) return HSMC_ERR_INVALID_ARG;
    for (int d = 0; d < 3; d++)
      if (!(conf[i][1 + d] >= 0.0 && conf[i][1 + d] <= bx.len[d])) return HSMC_ERR_OUT_OF_BOX;
  }
  const SysPtrs &s = b->sp[k];
  BATCH_CUDA(cudaMemcpyAsync(s.pos, conf, sizeof(double) * 4 * (size_t)n, cudaMemcpyHostToDevice, b->stream));
  for (int l = 0; l < 2; l++)
    BATCH_CUDA(cudaMemsetAsync(s.cnt[l], 0, sizeof(int) * (size_t)s.ncell_alloc, b->stream));
  BATCH_CUDA(cudaMemsetAsync(&s.st->status, 0, sizeof(int), b->stream));
  launch_build(s, -1, 0, b->stream);
  int e = batch_check(b);
  if (e) return e;
  DevState d;
  BATCH_CUDA(cudaMemcpy(&d, s.st, sizeof(DevState), cudaMemcpyDeviceToHost));
  if (d.status) return code_of(d.status);
  b->uploaded[k] = 1;
  return HSMC_OK;
}

int hsmc_batch_download_config(hsmc_batch *b, int k, double (*conf)[4], int n) {
  if (!b || k < 0 || k >= b->reps || !conf || n != b->sp[k].n) return HSMC_ERR_INVALID_ARG;
  BATCH_CUDA(cudaMemcpyAsync(conf, b->sp[k].pos, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost, b->stream));
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  return HSMC_OK;
}

int hsmc_batch_set_steps(hsmc_batch *b, const double *dr_max) {
  if (!b || !dr_max) return HSMC_ERR_INVALID_ARG;
  for (int k = 0; k < b->reps; k++)
    for (int d = 0; d < 3; d++)
      if (!(dr_max[k] >= 0 && dr_max[k] < b->hbox[k].len[d])) return HSMC_ERR_INVALID_ARG;
  BATCH_CUDA(cudaMemcpy2DAsync(&b->st[0].dr_max, sizeof(DevState), dr_max, sizeof(double), sizeof(double),
                               (size_t)b->reps, cudaMemcpyHostToDevice, b->stream));
  BATCH_CUDA(cudaStreamSynchronize(b->stream));
  for (int k = 0; k < b->reps; k++) b->prm[k].dr_max = dr_max[k];
  return HSMC_OK;
}

static void enqueue_batch_sweep(hsmc_batch *b, long long offset) {
  launch_build_batch(b->d_reps, b->d_nstart, b->reps, b->tot_n, offset, b->stream);
  const bool ordered = b->schedule == 3;
  if (ordered)
    for (const hsmc_batch::CapClass &cl : b->classes)
      launch_order_batch(cl.d_reps, cl.d_cstart, cl.n, cl.n_cells, cl.d_ocnt, cl.d_olist, cl.tot_groups, b->stream);
  for (int k = 0; k < 8; k++)
    for (size_t q = 0; q < b->classes.size(); q++) {
      const hsmc_batch::CapClass &cl = b->classes[q];
      // the first launch of the sweep's first pass clears the other layout
      const bool clear = q == 0;
      launch_move_pass_batch(cl.d_reps, cl.d_gstart, cl.d_ids, cl.n, cl.tot_groups, cl.cap, k, cl.group,
                             clear ? b->cnt[0] : nullptr, clear ? b->cnt[1] : nullptr, clear ? b->tot_cell : 0,
                             ordered ? cl.d_olist : nullptr, ordered ? cl.d_ocnt : nullptr, b->stream);
    }
}

// Packs the replicas of each cell capacity into bundles of at most `tile`
// active cells per lane group of a cluster (first fit, largest replica
// first, at most batch_persist_max_reps() replicas each; a larger replica is
// a bundle of its own), orders the bundles largest first, so the clusters
// that start first take the longest, and uploads the tables the persistent
// kernel reads.
static int build_bundles(hsmc_batch *b) {
  if (!b->bundles.empty() && b->bundled_cb == b->cluster_blocks && b->bundled_tile == b->tile) return HSMC_OK;
  free_bundles(b);
  const int max_reps = batch_persist_max_reps();
  for (int c : {8, 16, 32}) {
    std::vector<int> ks;
    for (int k = 0; k < b->reps; k++)
      if (b->sp[k].cap == c) ks.push_back(k);
    if (ks.empty()) continue;
    const long long target = (long long)b->tile * b->cluster_blocks * (128 / (c / 4));
    auto cells = [&](int k) { return (long long)b->hbox[k].ncell / 8; };
    std::stable_sort(ks.begin(), ks.end(), [&](int x, int y) { return cells(x) > cells(y); });
    std::vector<std::vector<int>> bun;
    std::vector<long long> load;
    for (int k : ks) {
      size_t j = 0;
      while (j < bun.size() && ((int)bun[j].size() >= max_reps || load[j] + cells(k) > target)) j++;
      if (j == bun.size()) {
        bun.emplace_back();
        load.push_back(0);
      }
      bun[j].push_back(k);
      load[j] += cells(k);
    }
    std::vector<size_t> order(bun.size());
    for (size_t j = 0; j < order.size(); j++) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return load[x] > load[y]; });
    std::vector<SysPtrs> sp;
    std::vector<int> ids, ns(1, 0), gs(1, 0), cs(1, 0), bs(1, 0);
    for (size_t j : order) {
      for (int k : bun[j]) {
        sp.push_back(b->sp[k]);
        ids.push_back(k);
        ns.push_back(ns.back() + b->sp[k].n);
        gs.push_back(gs.back() + b->hbox[k].ncell / 8);
        cs.push_back(cs.back() + b->hbox[k].ncell);
      }
      bs.push_back((int)sp.size());
    }
    hsmc_batch::Bundles q;
    q.cap = c;
    q.n_bundles = (int)bun.size();
    const size_t nr = sp.size();
    cudaError_t ce;
    if ((ce = cudaMalloc(&q.d_reps, sizeof(SysPtrs) * nr)) || (ce = cudaMalloc(&q.d_ids, sizeof(int) * nr)) ||
        (ce = cudaMalloc(&q.d_nstart, sizeof(int) * (nr + 1))) ||
        (ce = cudaMalloc(&q.d_gstart, sizeof(int) * (nr + 1))) ||
        (ce = cudaMalloc(&q.d_cstart, sizeof(int) * (nr + 1))) ||
        (ce = cudaMalloc(&q.d_bundle, sizeof(int) * bs.size())) ||
        (ce = cudaMemcpy(q.d_reps, sp.data(), sizeof(SysPtrs) * nr, cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_ids, ids.data(), sizeof(int) * nr, cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_nstart, ns.data(), sizeof(int) * (nr + 1), cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_gstart, gs.data(), sizeof(int) * (nr + 1), cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_cstart, cs.data(), sizeof(int) * (nr + 1), cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_bundle, bs.data(), sizeof(int) * bs.size(), cudaMemcpyHostToDevice))) {
      b->bundles.push_back(q);
      free_bundles(b);
      return cuda_fail(ce);
    }
    b->bundles.push_back(q);
  }
  b->bundled_cb = b->cluster_blocks;
  b->bundled_tile = b->tile;
  return HSMC_OK;
}

// The persistent schedule's launches for n_sweeps sweeps (one per cell
// capacity), captured once into a CUDA graph and kept while n_sweeps and the
// bundles stay the same.
static int ensure_persist_graph(hsmc_batch *b, int n_sweeps) {
  int e = build_bundles(b);
  if (e) return e;
  if (b->persist_graph && b->persist_graph_sweeps == n_sweeps) return HSMC_OK;
  if (b->persist_graph) cudaGraphExecDestroy(b->persist_graph);
  b->persist_graph = nullptr;
  cudaGraph_t g = nullptr;
  BATCH_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t le = cudaSuccess;
  for (const auto &q : b->bundles)
    if (le == cudaSuccess)
      le = launch_batch_persist(q.cap, q.d_reps, q.d_ids, q.d_nstart, q.d_gstart, q.d_cstart, q.d_bundle,
                                q.n_bundles, n_sweeps, b->cluster_blocks, b->stream);
  cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
  if (le != cudaSuccess || ce != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return cuda_fail(le != cudaSuccess ? le : ce);
  }
  ce = cudaGraphInstantiate(&b->persist_graph, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) {
    b->persist_graph = nullptr;
    return cuda_fail(ce);
  }
  b->persist_graph_sweeps = n_sweeps;
  return HSMC_OK;
}

// The grid schedule's tables per cell capacity: the class's replicas in
// batch order, with prefix sums of their particles, active cells and
// allocated cells, a parameter slot per replica and the barrier words.
static int build_grids(hsmc_batch *b) {
  if (!b->grids.empty()) return HSMC_OK;
  int dev = 0, sms = 0;
  BATCH_CUDA(cudaGetDevice(&dev));
  BATCH_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  for (int c : {8, 16, 32}) {
    std::vector<SysPtrs> sp;
    std::vector<int> ids, ns(1, 0), gs(1, 0), cs(1, 0);
    for (int k = 0; k < b->reps; k++) {
      if (b->sp[k].cap != c) continue;
      sp.push_back(b->sp[k]);
      ids.push_back(k);
      ns.push_back(ns.back() + b->sp[k].n);
      gs.push_back(gs.back() + b->hbox[k].ncell / 8);
      cs.push_back(cs.back() + b->hbox[k].ncell);
    }
    if (sp.empty()) continue;
    hsmc_batch::GridClass q;
    q.cap = c;
    q.n = (int)sp.size();
    q.blocks = batch_grid_blocks(c, sms);
    q.status = &sp[0].st->status;
    const size_t nr = sp.size();
    cudaError_t ce;
    if ((ce = cudaMalloc(&q.d_reps, sizeof(SysPtrs) * nr)) || (ce = cudaMalloc(&q.d_ids, sizeof(int) * nr)) ||
        (ce = cudaMalloc(&q.d_nstart, sizeof(int) * (nr + 1))) ||
        (ce = cudaMalloc(&q.d_gstart, sizeof(int) * (nr + 1))) ||
        (ce = cudaMalloc(&q.d_cstart, sizeof(int) * (nr + 1))) || (ce = cudaMalloc(&q.d_params, 16 * nr)) ||
        (ce = cudaMalloc(&q.d_bar, 8 * sizeof(unsigned))) ||
        (ce = cudaMemcpy(q.d_reps, sp.data(), sizeof(SysPtrs) * nr, cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_ids, ids.data(), sizeof(int) * nr, cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_nstart, ns.data(), sizeof(int) * (nr + 1), cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_gstart, gs.data(), sizeof(int) * (nr + 1), cudaMemcpyHostToDevice)) ||
        (ce = cudaMemcpy(q.d_cstart, cs.data(), sizeof(int) * (nr + 1), cudaMemcpyHostToDevice))) {
      b->grids.push_back(q);
      free_grids(b);
      return cuda_fail(ce);
    }
    b->grids.push_back(q);
    if (q.blocks <= 0) {
      free_grids(b);
      return HSMC_ERR_INVALID_ARG;
    }
  }
  return HSMC_OK;
}

int hsmc_batch_set_schedule(hsmc_batch *b, int schedule, int cluster_blocks, int tile) {
  if (!b || schedule < 0 || schedule > 3) return HSMC_ERR_INVALID_ARG;
  if (schedule == 2) {
    int dev = 0, coop = 0;
    BATCH_CUDA(cudaGetDevice(&dev));
    BATCH_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return HSMC_ERR_INVALID_ARG;
    BATCH_CUDA(prepare_batch_grid());
    int e = build_grids(b);
    if (e) return e;
  }
  if (schedule == 1) {
    if ((cluster_blocks != 1 && cluster_blocks != 2 && cluster_blocks != 4 && cluster_blocks != 8) || tile < 1 ||
        tile > 64)
      return HSMC_ERR_INVALID_ARG;
    int dev = 0, cl = 0;
    BATCH_CUDA(cudaGetDevice(&dev));
    BATCH_CUDA(cudaDeviceGetAttribute(&cl, cudaDevAttrClusterLaunch, dev));
    if (!cl) return HSMC_ERR_INVALID_ARG;
    BATCH_CUDA(prepare_batch_persist());
    for (const auto &cls : b->classes)
      if (batch_persist_max_clusters(cls.cap, cluster_blocks) <= 0) return HSMC_ERR_INVALID_ARG;
    if (cluster_blocks != b->cluster_blocks || tile != b->tile) free_bundles(b);
    b->cluster_blocks = cluster_blocks;
    b->tile = tile;
  }
  if ((schedule == 3) != (b->schedule == 3) && b->graph) {  // the flat launches' graph follows the order
    BATCH_CUDA(cudaStreamSynchronize(b->stream));
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  b->schedule = schedule;
  return HSMC_OK;
}

int hsmc_batch_get_schedule(hsmc_batch *b, int out[3]) {
  if (!b || !out) return HSMC_ERR_INVALID_ARG;
  out[0] = b->schedule;
  out[1] = b->cluster_blocks;
  out[2] = b->tile;
  return HSMC_OK;
}

int hsmc_batch_sweeps(hsmc_batch *b, int n_sweeps, uint64_t *counters) {
  if (!b || n_sweeps < 0) return HSMC_ERR_INVALID_ARG;
  for (int k = 0; k < b->reps; k++)
    if (!b->uploaded[k]) return HSMC_ERR_INVALID_ARG;
  const bool persist = b->schedule == 1 && n_sweeps > 0;
  const bool grid = b->schedule == 2 && n_sweeps > 0;
  if (persist) {
    int e = ensure_persist_graph(b, n_sweeps);
    if (e) return e;
  }
  if (grid) {
    int e = build_grids(b);
    if (e) return e;
  }
  if (!persist && !grid && !b->graph) {
    cudaGraph_t g = nullptr;
    BATCH_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < kBatchGraphSweeps; s++) enqueue_batch_sweep(b, s);
    launch_advance_batch(b->d_reps, b->reps, kBatchGraphSweeps, b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) return cuda_fail(e);
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      b->graph = nullptr;
      return cuda_fail(e);
    }
  }
  // counters (acc .. scan_mask) and status of every replica
  BATCH_CUDA(cudaMemset2DAsync(&b->st[0].acc, sizeof(DevState), 0, offsetof(DevState, dr_max) - offsetof(DevState, acc),
                               (size_t)b->reps, b->stream));
  BATCH_CUDA(cudaMemset2DAsync(&b->st[0].status, sizeof(DevState), 0, sizeof(int), (size_t)b->reps, b->stream));
  BATCH_CUDA(cudaEventRecord(b->ev0, b->stream));
  if (persist) {
    BATCH_CUDA(cudaGraphLaunch(b->persist_graph, b->stream));
  } else if (grid) {
    for (const auto &q : b->grids) {
      BATCH_CUDA(cudaMemsetAsync(q.d_bar, 0, 8 * sizeof(unsigned), b->stream));
      BATCH_CUDA(launch_batch_grid(q.cap, q.d_reps, q.d_ids, q.d_nstart, q.d_gstart, q.d_cstart, q.d_params, q.d_bar,
                                   reinterpret_cast<int *>(q.d_bar + 2), q.d_bar + 4, q.status, q.n, n_sweeps,
                                   q.blocks, b->stream));
    }
  } else {
    int done = 0;
    while (n_sweeps - done >= kBatchGraphSweeps) {
      BATCH_CUDA(cudaGraphLaunch(b->graph, b->stream));
      done += kBatchGraphSweeps;
    }
    const int rest = n_sweeps - done;
    for (int s = 0; s < rest; s++) enqueue_batch_sweep(b, s);
    if (rest > 0) launch_advance_batch(b->d_reps, b->reps, rest, b->stream);
  }
  BATCH_CUDA(cudaEventRecord(b->ev1, b->stream));
  int e = batch_check(b);
  if (e) return e;
  float ms = 0.f;
  BATCH_CUDA(cudaEventElapsedTime(&ms, b->ev0, b->ev1));
  b->last_ms = ms;
  std::vector<DevState> st;
  const int status = batch_status(b, st);
  if (counters) {
    for (int k = 0; k < b->reps; k++) {
      const uint64_t moves = (uint64_t)b->sp[k].n * (uint64_t)n_sweeps;
      uint64_t *c = counters + 6 * (size_t)k;
      c[HSMC_CNT_MOVES] = moves;
      c[HSMC_CNT_ACCEPTED] = st[k].acc;
      c[HSMC_CNT_REJECTED] = moves - st[k].acc;
      c[HSMC_CNT_VOL_MOVES] = c[HSMC_CNT_VOL_ACCEPTED] = c[HSMC_CNT_VOL_REJECTED] = 0;
    }
  }
  return status;
}

// Times the flat schedule, the grid schedule and the cluster schedule with
// every cluster size (1, 2, 4, 8 blocks) and tile (1, 2, 4 active cells per
// lane group and bundle), each over sweeps_per_variant sweeps after an
// untimed call of 8, and keeps the fastest.  The chain is the same for all
// of them.
int hsmc_batch_autotune(hsmc_batch *b, int sweeps_per_variant, int out[3]) {
  if (!b || sweeps_per_variant <= 0) return HSMC_ERR_INVALID_ARG;
  struct V {
    int s, cb, tile;
  };
  std::vector<V> vs{{0, b->cluster_blocks, b->tile}, {3, b->cluster_blocks, b->tile}, {2, b->cluster_blocks, b->tile}};
  for (int cb : {1, 2, 4, 8})
    for (int tile : {1, 2, 4}) vs.push_back({1, cb, tile});
  V best = vs[0];
  double best_ms = 1e300;
  for (const V &v : vs) {
    if (hsmc_batch_set_schedule(b, v.s, v.cb, v.tile) != HSMC_OK) continue;
    int e = hsmc_batch_sweeps(b, kBatchGraphSweeps, nullptr);
    if (!e) e = hsmc_batch_sweeps(b, sweeps_per_variant, nullptr);
    if (e) return e;
    if (b->last_ms < best_ms) {
      best_ms = b->last_ms;
      best = v;
    }
  }
  int e = hsmc_batch_set_schedule(b, best.s, best.cb, best.tile);
  if (e) return e;
  if (best.s != 1 && (b->cluster_blocks != best.cb || b->tile != best.tile)) {
    // the flat or grid launches won (either order): keep the cluster shape the batch had before
    free_bundles(b);
    b->cluster_blocks = best.cb;
    b->tile = best.tile;
  }
  return out ? hsmc_batch_get_schedule(b, out) : HSMC_OK;
}

int hsmc_batch_pressv(hsmc_batch *b, double dr, double rmax, int nbins, uint64_t *counts) {
  if (!b || !counts || nbins <= 0 || !(dr > 0) || !(rmax > 1.0)) return HSMC_ERR_INVALID_ARG;
  for (int k = 0; k < b->reps; k++)
    if (!b->uploaded[k]) return HSMC_ERR_INVALID_ARG;
  const size_t need = (size_t)nbins * b->reps;
  if (need > b->hist_bins) {
    cudaFree(b->hist);
    b->hist = nullptr;
    b->hist_bins = 0;
    BATCH_CUDA(cudaMalloc(&b->hist, sizeof(unsigned long long) * need));
    b->hist_bins = need;
  }
  BATCH_CUDA(cudaMemsetAsync(b->hist, 0, sizeof(unsigned long long) * need, b->stream));
  BATCH_CUDA(cudaMemset2DAsync(&b->st[0].status, sizeof(DevState), 0, sizeof(int), (size_t)b->reps, b->stream));
  launch_pair_hist_batch(b->d_reps, b->reps, b->max_n, dr, rmax, nbins, b->hist, b->stream);
  int e = batch_check(b);
  if (e) return e;
  BATCH_CUDA(cudaMemcpy(counts, b->hist, sizeof(uint64_t) * need, cudaMemcpyDeviceToHost));
  std::vector<DevState> st;
  return batch_status(b, st);
}

int hsmc_batch_last_timing(hsmc_batch *b, double *total_ms) {
  if (!b || !total_ms) return HSMC_ERR_INVALID_ARG;
  *total_ms = b->last_ms;
  return HSMC_OK;
}

}  // extern "C"
