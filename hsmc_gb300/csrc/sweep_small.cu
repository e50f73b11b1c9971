// Whole checkerboard sweeps of a small system in one block (the "one block"
// schedule).  The eight launches per sweep of the pass-barrier schedule cost
// more than the work for a few thousand spheres: launch gaps dominate a
// sweep of N = 256 to 4000.  Here one launch runs every sweep of a call with
// the system in shared memory: FP64 positions, their grid coordinates, and a
// cell list by counting sort (ids ascending within a cell), rebuilt on each
// sweep's shifted grid; colour passes are separated by block barriers.
//
// The chain is the pass-barrier schedule's bit for bit: the same grid
// shift and colour order per sweep (k_build), the same Philox counters per
// cell and trial, the particle of rank floor(u n) by id, the same FP64
// proposal and confinement test, and overlap decisions that are the
// reference's FP64 test (single precision decides only outside the guard
// band).  Up to 128 active cells per pass, a group of 32, 16, 8 or 4 lanes
// per cell makes the cell's trials one after another and a pass has one
// block barrier, at its end.  Above that a pass runs in rounds, round t
// making trial t of every active cell that has one: one thread per cell
// draws and proposes (so one warp's FP64 sequence serves 32 cells: GB300's
// FP64 pipe is busy per warp instruction), then one warp per cell screens
// it, lane k on neighbour cell k of the 27, and the cell's thread applies
// an accepted move at the start of the next round.  Either way a cell's
// trials stay in order; its neighbours are of other colours, so no other
// cell writes what it reads.
//
// NpT sweeps add vol_move after the passes (src/moves.c:83-153): one thread
// proposes, the block scans every particle's neighbourhood at the scaled
// distances, one thread decides and rebuilds the box, and the block rescales
// the positions; the box lives in shared memory for the launch.  The
// arithmetic is engine.cuh's, shared with the volume-move kernels, so the
// chain is the one of the eight-launch sweep followed by those kernels.
// Cavity runs add their cavity stage after the passes, warp 0 making the
// trials with cavity.cuh's loop against the shared-memory cell list.
#include "cavity.cuh"

namespace hsmc {

namespace {

// Threads of the block: 512 leave each 128 registers, which the lane groups'
// trial loop needs without spilling; the rounds below take up to one active
// cell per thread.
constexpr int kSmallThreads = 512;

struct SmallSweepSm {
  double *x, *y, *z;     // N positions
  double *px, *py, *pz;  // per active cell: this round's trial position
  float *tx, *ty, *tz;   // N grid coordinates on the current sweep's grid
  float *ux, *uy, *uz;   // per active cell: the trial's grid coordinates
  uint32_t *fill;        // ncell counts, then scatter cursors
  uint16_t *start;       // ncell + 1 offsets into ids
  uint16_t *ids;         // N particle ids by cell, ascending within a cell
  uint16_t *tid_;        // per active cell: the trial's particle
  uint8_t *state;        // per active cell: 0 no trial to screen, 1 screen it, 2 overlap found
  uint4 *draws;          // per active cell and trial (cap of them): the pass's Philox draws
};

__device__ __forceinline__ SmallSweepSm small_sweep_sm(unsigned char *raw, int n, int ncell, int na, int cap) {
  SmallSweepSm m;
  m.draws = reinterpret_cast<uint4 *>(raw);  // 16-byte aligned first
  raw += 16 * (size_t)na * cap;
  m.x = reinterpret_cast<double *>(raw);
  m.y = m.x + n;
  m.z = m.y + n;
  m.px = m.z + n;
  m.py = m.px + na;
  m.pz = m.py + na;
  m.tx = reinterpret_cast<float *>(m.pz + na);
  m.ty = m.tx + n;
  m.tz = m.ty + n;
  m.ux = m.tz + n;
  m.uy = m.ux + na;
  m.uz = m.uy + na;
  m.fill = reinterpret_cast<uint32_t *>(m.uz + na);
  m.start = reinterpret_cast<uint16_t *>(m.fill + ncell);
  m.ids = m.start + (ncell + 1);
  m.tid_ = m.ids + n;
  m.state = reinterpret_cast<uint8_t *>(m.tid_ + na);
  return m;
}

// Exclusive scan of fill[0..ncell) into start (a contiguous chunk per
// thread, then a block scan of the chunk sums).
__device__ void scan_cells(const SmallSweepSm &m, int ncell, int n) {
  const int tid = (int)threadIdx.x, nt = (int)blockDim.x;
  const int per = (ncell + nt - 1) / nt;
  const int c0 = tid * per, c1 = min(c0 + per, ncell);
  uint32_t sum = 0;
  for (int c = c0; c < c1; c++) sum += m.fill[c];
  const int lane = tid & 31, w = tid >> 5;
  uint32_t inc = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  __shared__ uint32_t wsum[32];
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t v = lane < (nt >> 5) ? wsum[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    wsum[lane] = v;
  }
  __syncthreads();
  uint32_t run = (w ? wsum[w - 1] : 0u) + inc - sum;
  for (int c = c0; c < c1; c++) {
    m.start[c] = (uint16_t)run;
    run += m.fill[c];
  }
  if (tid == nt - 1) m.start[ncell] = (uint16_t)n;
  __syncthreads();
}

// A coordinate scaled by sf and wrapped once into [0, L] (src/moves.c:133-140).
__device__ __forceinline__ double scale_wrap(double x, double sf, double len) {
  double v = __dmul_rn(x, sf);
  if (gt_pos(v, len)) v = __dsub_rn(v, len);
  else if (lt_zero(v)) v = __dadd_rn(v, len);
  return v;
}

// One colour pass of up to 128 active cells by lane groups (gsz lanes per
// cell), for k_sweep_small.
__device__ __forceinline__ void small_pass_groups(const SmallSweepSm &m, const Box &sb, const float *sh_s, int colour,
                                               unsigned long long seq, int gsz, int n_active, int cap, int frozen,
                                               unsigned long long seed, double dr, unsigned &acc, unsigned &rej_o,
                                               unsigned &rej_b) {
  const int tid = (int)threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = (int)blockDim.x >> 5;
  const int nc[3] = {sb.nc[0], sb.nc[1], sb.nc[2]};
  const int hx = nc[0] >> 1, hy = nc[1] >> 1;
  const double len[3] = {sb.len[0], sb.len[1], sb.len[2]};
  const double *half = sb.half;
  const float L32[3] = {sb.len32[0], sb.len32[1], sb.len32[2]};
  const float iw[3] = {sb.inv_w32[0], sb.inv_w32[1], sb.inv_w32[2]};
  const float sh[3] = {sh_s[0], sh_s[1], sh_s[2]};
  const float lo = 1.0f - sb.band, hi = 1.0f + sb.band;
  const int gl = lane & (gsz - 1), gpw = 32 / gsz;
  const unsigned gmask = gsz == 32 ? 0xffffffffu : (((1u << gsz) - 1u) << (lane - gl));
  for (int a = wid * gpw + lane / gsz; a < n_active; a += nw * gpw) {  // the same in the group's lanes
    const int ax = a % hx, ayz = a / hx, ay = ayz % hy, az = ayz / hy;
    const int ix = 2 * ax + (colour & 1), iy = 2 * ay + ((colour >> 1) & 1), iz = 2 * az + ((colour >> 2) & 1);
    const int c = ix + nc[0] * (iy + nc[1] * iz);
    const int b = m.start[c];
    int cn = m.start[c + 1] - b;
    if (cn > cap) cn = 0;  // an overfull cell was flagged above
    U32x4 dl = {0u, 0u, 0u, 0u};
    if (gl < cn) dl = draw4(seed, (uint32_t)gl, (uint32_t)c, seq, TAG_MOVE);
    for (int t = 0; t < cn; t++) {
      U32x4 r;
      if (t < gsz) {
        r.x = __shfl_sync(gmask, dl.x, t, gsz);
        r.y = __shfl_sync(gmask, dl.y, t, gsz);
        r.z = __shfl_sync(gmask, dl.z, t, gsz);
        r.w = __shfl_sync(gmask, dl.w, t, gsz);
      } else {
        r = draw4(seed, (uint32_t)t, (uint32_t)c, seq, TAG_MOVE);
      }
      const int id = m.ids[b + (int)__umulhi(r.x, (unsigned)cn)];
      if (id < frozen) continue;  // a cavity is moved by the cavity stage
      const int ag = gl < 3 ? gl : 2;  // this lane's axis
      const double xa = ag == 0 ? m.x[id] : (ag == 1 ? m.y[id] : m.z[id]);
      const double va = propose_axis(xa, centred_offset(ag == 0 ? r.y : (ag == 1 ? r.z : r.w)), dr,
                                     ag == 0 ? len[0] : (ag == 1 ? len[1] : len[2]));
      int ca;
      float ua;
      axis_cell(__double2float_rn(va), ag == 0 ? sh[0] : (ag == 1 ? sh[1] : sh[2]),
                ag == 0 ? L32[0] : (ag == 1 ? L32[1] : L32[2]), ag == 0 ? iw[0] : (ag == 1 ? iw[1] : iw[2]),
                ag == 0 ? nc[0] : (ag == 1 ? nc[1] : nc[2]), ca, ua);
      const double nx = __shfl_sync(gmask, va, 0, gsz), ny = __shfl_sync(gmask, va, 1, gsz),
                   nz = __shfl_sync(gmask, va, 2, gsz);
      const float ux = __shfl_sync(gmask, ua, 0, gsz), uy = __shfl_sync(gmask, ua, 1, gsz),
                  uz = __shfl_sync(gmask, ua, 2, gsz);
      const int c0 = __shfl_sync(gmask, ca, 0, gsz), c1 = __shfl_sync(gmask, ca, 1, gsz),
                c2 = __shfl_sync(gmask, ca, 2, gsz);
      if (c0 != ix || c1 != iy || c2 != iz) {
        if (gl == 0) rej_b++;  // the move would leave the active cell
        continue;
      }
      bool ov = false;
      for (int k = gl; k < 27 && !ov; k += gsz) {
        int jx = ix + k % 3 - 1, jy = iy + (k / 3) % 3 - 1, jz = iz + k / 9 - 1;
        float imx = 0.f, imy = 0.f, imz = 0.f;
        if (jx < 0) { jx += nc[0]; imx = -L32[0]; } else if (jx >= nc[0]) { jx -= nc[0]; imx = L32[0]; }
        if (jy < 0) { jy += nc[1]; imy = -L32[1]; } else if (jy >= nc[1]) { jy -= nc[1]; imy = L32[1]; }
        if (jz < 0) { jz += nc[2]; imz = -L32[2]; } else if (jz >= nc[2]) { jz -= nc[2]; imz = L32[2]; }
        const int nb = jx + nc[0] * (jy + nc[1] * jz);
        const int qe = m.start[nb + 1];
        for (int q = m.start[nb]; q < qe && !ov; q++) {
          const int j = m.ids[q];
          if (j == id) continue;
          const float dx = ux - __fadd_rn(m.tx[j], imx), dy = uy - __fadd_rn(m.ty[j], imy),
                      dz = uz - __fadd_rn(m.tz[j], imz);
          const float r2 = dx * dx + dy * dy + dz * dz;
          if (r2 < lo) ov = true;
          else if (r2 <= hi) ov = ref_r2(nx, ny, nz, m.x[j], m.y[j], m.z[j], len, half) < 1.0;
        }
      }
      if (__ballot_sync(gmask, ov) != 0u) {
        if (gl == 0) rej_o++;
      } else {
        if (gl == 0) {
          m.x[id] = nx;
          m.y[id] = ny;
          m.z[id] = nz;
          m.tx[id] = ux;
          m.ty[id] = uy;
          m.tz[id] = uz;
          acc++;
        }
        __syncwarp(gmask);  // the next trial reads the move
      }
    }
  }
}

template <bool CAV>
__global__ void __launch_bounds__(kSmallThreads) k_sweep_small(SysPtrs p, int n_sweeps, int npt, double margin) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float sh_s[3];
  __shared__ int perm_s[8];
  __shared__ Box sb;         // the box, which a volume move may change
  __shared__ double v_new, v_ratio, v_sf, v_u;
  __shared__ int v_ov, v_acc;
  DevState *st = p.st;
  const int n = p.n, cap = p.cap;
  // array sizes for the largest grid the context allocated (an NpT box can grow)
  const SmallSweepSm m = small_sweep_sm(smem_raw, n, p.ncell_alloc, p.ncell_alloc / 8, cap);
  __shared__ int max_cn[8];  // per colour: the most trials any of its cells makes
  const int tid = (int)threadIdx.x, nt = (int)blockDim.x;
  if (tid == 0) sb = *p.box;
  const double dr = st->dr_max;
  const unsigned long long seed = st->seed, s0 = st->sweep_base;
  const int frozen = st->frozen;
  const bool cavity = CAV && frozen == 2 && st->cav_trials > 0;
  for (int i = tid; i < n; i += nt) load_xyz(p.pos, i, m.x[i], m.y[i], m.z[i]);
  unsigned acc = 0, rej_o = 0, rej_b = 0;
  unsigned long long vmoves = 0, vacc = 0, cdone = 0, cacc = 0;
  const int lane = tid & 31, wid = tid >> 5, nw = nt >> 5;
  __syncthreads();

  for (int sw = 0; sw < n_sweeps; sw++) {
    const unsigned long long s = s0 + (unsigned long long)sw;
    // this sweep's box and grid
    const int nc[3] = {sb.nc[0], sb.nc[1], sb.nc[2]};
    const int ncell = sb.ncell, hx = nc[0] >> 1, hy = nc[1] >> 1;
    const int n_active = hx * hy * (nc[2] >> 1);
    double len[3], half[3];
    float L32[3], iw[3];
    for (int d = 0; d < 3; d++) {
      len[d] = sb.len[d];
      half[d] = sb.half[d];
      L32[d] = sb.len32[d];
      iw[d] = sb.inv_w32[d];
    }
    const float lo = 1.0f - sb.band, hi = 1.0f + sb.band;
    // the sweep's grid shift and colour order, as k_build draws them
    if (tid == 0) {
      const U32x4 rs = draw4(seed, 0u, 0u, s, TAG_SHIFT);
      sh_s[0] = __fmul_rn(__uint2float_rn(rs.x >> 8) * 5.9604644775390625e-08f, sb.w32[0]);
      sh_s[1] = __fmul_rn(__uint2float_rn(rs.y >> 8) * 5.9604644775390625e-08f, sb.w32[1]);
      sh_s[2] = __fmul_rn(__uint2float_rn(rs.z >> 8) * 5.9604644775390625e-08f, sb.w32[2]);
      int perm[8] = {0, 1, 2, 3, 4, 5, 6, 7};
      const U32x4 ra = draw4(seed, 0u, 0u, s, TAG_PERM), rb = draw4(seed, 1u, 0u, s, TAG_PERM);
      const uint32_t r[7] = {ra.x, ra.y, ra.z, ra.w, rb.x, rb.y, rb.z};
      for (int k = 7; k >= 1; k--) {  // Fisher-Yates
        const int j = (int)__umulhi(r[7 - k], (unsigned)(k + 1));
        const int tmp = perm[k];
        perm[k] = perm[j];
        perm[j] = tmp;
      }
      for (int k = 0; k < 8; k++) perm_s[k] = perm[k];
    }
    for (int c = tid; c < ncell; c += nt) m.fill[c] = 0u;
    __syncthreads();
    const float sh[3] = {sh_s[0], sh_s[1], sh_s[2]};
    // cells of the shifted grid: counting sort
    for (int i = tid; i < n; i += nt) {
      int cx, cy, cz;
      axis_cell(__double2float_rn(m.x[i]), sh[0], L32[0], iw[0], nc[0], cx, m.tx[i]);
      axis_cell(__double2float_rn(m.y[i]), sh[1], L32[1], iw[1], nc[1], cy, m.ty[i]);
      axis_cell(__double2float_rn(m.z[i]), sh[2], L32[2], iw[2], nc[2], cz, m.tz[i]);
      atomicAdd(m.fill + cx + nc[0] * (cy + nc[1] * cz), 1u);
    }
    __syncthreads();
    if (tid < 8) max_cn[tid] = 0;
    __syncthreads();
    for (int c = tid; c < ncell; c += nt) {
      const uint32_t k = m.fill[c];
      if (k > (uint32_t)cap) {
        atomicOr(&st->status, ST_CELL_OVERFLOW);
      } else if (k > 0) {
        const int cx = c % nc[0], cyz = c / nc[0], cy = cyz % nc[1], cz = cyz / nc[1];
        atomicMax(max_cn + cell_colour(cx, cy, cz), (int)k);
      }
    }
    scan_cells(m, ncell, n);
    for (int c = tid; c < ncell; c += nt) m.fill[c] = 0u;
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
      int cx, cy, cz;
      float t;
      axis_cell(__double2float_rn(m.x[i]), sh[0], L32[0], iw[0], nc[0], cx, t);
      axis_cell(__double2float_rn(m.y[i]), sh[1], L32[1], iw[1], nc[1], cy, t);
      axis_cell(__double2float_rn(m.z[i]), sh[2], L32[2], iw[2], nc[2], cz, t);
      const int c = cx + nc[0] * (cy + nc[1] * cz);
      m.ids[m.start[c] + atomicAdd(m.fill + c, 1u)] = (uint16_t)i;
    }
    __syncthreads();
    for (int c = tid; c < ncell; c += nt) {  // ids ascending within each cell
      const int b = m.start[c], e = m.start[c + 1];
      for (int a = b + 1; a < e; a++) {
        const uint16_t v = m.ids[a];
        int q = a - 1;
        while (q >= b && m.ids[q] > v) {
          m.ids[q + 1] = m.ids[q];
          q--;
        }
        m.ids[q + 1] = v;
      }
    }
    __syncthreads();

    // Up to 128 active cells per pass (up to 8 lane groups a warp): a group of
    // lanes per cell makes the cell's trials one after another, with no
    // block barrier until the pass ends.  Its lane t draws trial t, three
    // lanes make the FP64 proposal (an axis each), and the lanes screen the
    // 27 neighbour cells and the cell's own; the group's first lane applies
    // an accepted move.  The cells of a colour are independent, so this is
    // the chain of the rounds below (which serve larger systems), trial for
    // trial.
    const int gsz = n_active > 128 ? 0 : (n_active <= nw ? 32 : (n_active <= 2 * nw ? 16 : (n_active <= 4 * nw ? 8 : 4)));
    for (int pass = 0; gsz > 0 && pass < 8; pass++) {
      small_pass_groups(m, sb, sh_s, perm_s[pass], s * 8ull + (unsigned long long)pass, gsz, n_active, cap, frozen,
                        seed, dr, acc, rej_o, rej_b);
      __syncthreads();  // every move of the pass is seen by the next
    }

    for (int pass = 0; gsz == 0 && pass < 8; pass++) {
      const int colour = perm_s[pass];
      const unsigned long long seq = s * 8ull + (unsigned long long)pass;
      // this thread's cell (n_active <= blockDim.x)
      const bool own = tid < n_active;
      int ix = 0, iy = 0, iz = 0, c = 0, b = 0, cn = 0;
      if (own) {
        const int ax = tid % hx, ayz = tid / hx, ay = ayz % hy, az = ayz / hy;
        ix = 2 * ax + (colour & 1);
        iy = 2 * ay + ((colour >> 1) & 1);
        iz = 2 * az + ((colour >> 2) & 1);
        c = ix + nc[0] * (iy + nc[1] * iz);
        b = m.start[c];
        cn = m.start[c + 1] - b;
        if (cn > cap) cn = 0;  // an overfull cell was flagged above
      }
      const int rounds = max_cn[colour];
      // every trial's draws of the pass at once, one thread per (cell,
      // trial), off the rounds' critical path
      for (int k = tid; k < n_active * rounds; k += nt) {
        const int a = k % n_active, t = k / n_active;
        const int ax = a % hx, ayz = a / hx, ay = ayz % hy, az = ayz / hy;
        const int ca = (2 * ax + (colour & 1)) + nc[0] * ((2 * ay + ((colour >> 1) & 1)) + nc[1] * (2 * az + ((colour >> 2) & 1)));
        const U32x4 d = draw4(seed, (uint32_t)t, (uint32_t)ca, seq, TAG_MOVE);
        m.draws[a * cap + t] = make_uint4(d.x, d.y, d.z, d.w);
      }
      __syncthreads();
      for (int round = 0; round <= rounds; round++) {
        // the cell's thread: apply the previous round's accepted move, then
        // draw and propose this round's trial
        if (own) {
          const int st_prev = round > 0 ? m.state[tid] : 0;
          if (st_prev == 1) {
            const int id = m.tid_[tid];
            m.x[id] = m.px[tid];
            m.y[id] = m.py[tid];
            m.z[id] = m.pz[tid];
            m.tx[id] = m.ux[tid];
            m.ty[id] = m.uy[tid];
            m.tz[id] = m.uz[tid];
            acc++;
          } else if (st_prev == 2) {
            rej_o++;
          }
          uint8_t state = 0;
          if (round < cn) {
            const uint4 r = m.draws[tid * cap + round];
            const int id = m.ids[b + (int)__umulhi(r.x, (unsigned)cn)];
            if (id >= frozen) {  // a cavity is moved by the cavity stage
              const double nx = propose_axis(m.x[id], centred_offset(r.y), dr, len[0]);
              const double ny = propose_axis(m.y[id], centred_offset(r.z), dr, len[1]);
              const double nz = propose_axis(m.z[id], centred_offset(r.w), dr, len[2]);
              int c0, c1, c2;
              float ux, uy, uz;
              axis_cell(__double2float_rn(nx), sh[0], L32[0], iw[0], nc[0], c0, ux);
              axis_cell(__double2float_rn(ny), sh[1], L32[1], iw[1], nc[1], c1, uy);
              axis_cell(__double2float_rn(nz), sh[2], L32[2], iw[2], nc[2], c2, uz);
              if (c0 != ix || c1 != iy || c2 != iz) {
                rej_b++;  // the move would leave the active cell
              } else {
                m.px[tid] = nx;
                m.py[tid] = ny;
                m.pz[tid] = nz;
                m.ux[tid] = ux;
                m.uy[tid] = uy;
                m.uz[tid] = uz;
                m.tid_[tid] = (uint16_t)id;
                state = 1;
              }
            }
          }
          m.state[tid] = state;
        }
        __syncthreads();
        if (round == rounds) break;
        // one warp per cell with a trial: lane k screens neighbour cell k
        for (int ac = wid; ac < n_active; ac += nw) {
          if (m.state[ac] != 1) continue;
          const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
          const int jx0 = 2 * ax + (colour & 1), jy0 = 2 * ay + ((colour >> 1) & 1), jz0 = 2 * az + ((colour >> 2) & 1);
          const int id = m.tid_[ac];
          const float ux = m.ux[ac], uy = m.uy[ac], uz = m.uz[ac];
          bool ov = false;
          if (lane < 27) {
            int jx = jx0 + lane % 3 - 1, jy = jy0 + (lane / 3) % 3 - 1, jz = jz0 + lane / 9 - 1;
            float imx = 0.f, imy = 0.f, imz = 0.f;
            if (jx < 0) { jx += nc[0]; imx = -L32[0]; } else if (jx >= nc[0]) { jx -= nc[0]; imx = L32[0]; }
            if (jy < 0) { jy += nc[1]; imy = -L32[1]; } else if (jy >= nc[1]) { jy -= nc[1]; imy = L32[1]; }
            if (jz < 0) { jz += nc[2]; imz = -L32[2]; } else if (jz >= nc[2]) { jz -= nc[2]; imz = L32[2]; }
            const int nb = jx + nc[0] * (jy + nc[1] * jz);
            const int qe = m.start[nb + 1];
            for (int q = m.start[nb]; q < qe && !ov; q++) {
              const int j = m.ids[q];
              if (j == id) continue;
              const float dx = ux - __fadd_rn(m.tx[j], imx), dy = uy - __fadd_rn(m.ty[j], imy),
                          dz = uz - __fadd_rn(m.tz[j], imz);
              const float r2 = dx * dx + dy * dy + dz * dz;
              if (r2 < lo) ov = true;
              else if (r2 <= hi)
                ov = ref_r2(m.px[ac], m.py[ac], m.pz[ac], m.x[j], m.y[j], m.z[j], len, half) < 1.0;
            }
          }
          if (__any_sync(0xffffffffu, ov) && lane == 0) m.state[ac] = 2;
        }
        __syncthreads();
      }
      __syncthreads();
    }
    if (CAV && cavity) {  // the sweep's cavity trials (cavity.cu's stage)
      if (wid == 0) {
        double cav[2][3] = {{m.x[0], m.y[0], m.z[0]}, {m.x[1], m.y[1], m.z[1]}};
        const int ox = lane % 3 - 1, oy = (lane / 3) % 3 - 1, oz = lane / 9 - 1;
        auto overlaps = [&](const double *nw) -> bool {
          bool ov = false;
          if (lane < 27) {
            int ci[3];
            float t[3];
            axis_cell(__double2float_rn(nw[0]), sh[0], L32[0], iw[0], nc[0], ci[0], t[0]);
            axis_cell(__double2float_rn(nw[1]), sh[1], L32[1], iw[1], nc[1], ci[1], t[1]);
            axis_cell(__double2float_rn(nw[2]), sh[2], L32[2], iw[2], nc[2], ci[2], t[2]);
            int jx = ci[0] + ox, jy = ci[1] + oy, jz = ci[2] + oz;
            float imx = 0.f, imy = 0.f, imz = 0.f;
            if (jx < 0) { jx += nc[0]; imx = -L32[0]; } else if (jx >= nc[0]) { jx -= nc[0]; imx = L32[0]; }
            if (jy < 0) { jy += nc[1]; imy = -L32[1]; } else if (jy >= nc[1]) { jy -= nc[1]; imy = L32[1]; }
            if (jz < 0) { jz += nc[2]; imz = -L32[2]; } else if (jz >= nc[2]) { jz -= nc[2]; imz = L32[2]; }
            const int nb = jx + nc[0] * (jy + nc[1] * jz);
            const int qe = m.start[nb + 1];
            for (int q = m.start[nb]; q < qe && !ov; q++) {
              const int j = m.ids[q];
              if (j < 2) continue;  // the cavities do not overlap each other
              const float dx = t[0] - __fadd_rn(m.tx[j], imx), dy = t[1] - __fadd_rn(m.ty[j], imy),
                          dz = t[2] - __fadd_rn(m.tz[j], imz);
              const float r2 = dx * dx + dy * dy + dz * dz;
              if (r2 < lo) ov = true;
              else if (r2 <= hi) ov = ref_r2(nw[0], nw[1], nw[2], m.x[j], m.y[j], m.z[j], len, half) < 1.0;
            }
          }
          return __any_sync(0xffffffffu, ov);
        };
        auto accept = [&](int w, const double *nw) {
          if (lane == 0) {
            m.x[w] = nw[0];
            m.y[w] = nw[1];
            m.z[w] = nw[2];
          }
        };
        cavity_trials(st, s, cav, len, half, overlaps, accept, nullptr, 0, nullptr, &st->status, cdone, cacc);
      }
      __syncthreads();
    }
    if (npt) {
      // vol_move: propose (one thread)
      if (tid == 0) {
        const U32x4 r = draw4(seed, 0u, 0u, s, TAG_VOLUME);
        double vn, ra, sf;
        vol_proposal(sb.vol, r.x, st->dv_max, vn, ra, sf);
        v_new = vn;
        v_ratio = ra;
        v_sf = sf;
        v_u = open_unit(r.y);
        v_ov = 0;
        v_acc = 0;
        vmoves++;
      }
      __syncthreads();
      const double sf = v_sf;
      if (vol_scan_needed(sf, sb.len)) {  // an expansion clear of 1 is not scanned
        // check_overlap(i, sf, sf, sf) for every i (src/moves.c:104-112)
        const float reach = (float)(1.0 / sf) + 1e-3f;
        int k[3];
        for (int d = 0; d < 3; d++) {
          k[d] = (int)ceilf(reach * iw[d] * 1.0001f);
          if (2 * k[d] + 1 > nc[d]) k[d] = -1;
        }
        for (int i = tid; i < n; i += nt) {
          if (*(volatile int *)&v_ov) break;
          int ci[3];
          float xs[3];
          axis_cell(__double2float_rn(m.x[i]), sh[0], L32[0], iw[0], nc[0], ci[0], xs[0]);
          axis_cell(__double2float_rn(m.y[i]), sh[1], L32[1], iw[1], nc[1], ci[1], xs[1]);
          axis_cell(__double2float_rn(m.z[i]), sh[2], L32[2], iw[2], nc[2], ci[2], xs[2]);
          bool ov = false;
          for (int a = (k[2] < 0 ? 0 : -k[2]); !ov && a <= (k[2] < 0 ? nc[2] - 1 : k[2]); a++) {
            const int cz = k[2] < 0 ? a : (ci[2] + a + nc[2]) % nc[2];
            for (int b2 = (k[1] < 0 ? 0 : -k[1]); !ov && b2 <= (k[1] < 0 ? nc[1] - 1 : k[1]); b2++) {
              const int cy = k[1] < 0 ? b2 : (ci[1] + b2 + nc[1]) % nc[1];
              for (int e = (k[0] < 0 ? 0 : -k[0]); !ov && e <= (k[0] < 0 ? nc[0] - 1 : k[0]); e++) {
                const int cx = k[0] < 0 ? e : (ci[0] + e + nc[0]) % nc[0];
                const int cc = cx + nc[0] * (cy + nc[1] * cz);
                const int qe = m.start[cc + 1];
                for (int q = m.start[cc]; q < qe && !ov; q++) {
                  const int j = m.ids[q];
                  if (j == i) continue;
                  float dx = xs[0] - m.tx[j], dy = xs[1] - m.ty[j], dz = xs[2] - m.tz[j];
                  dx -= L32[0] * rintf(dx / L32[0]);
                  dy -= L32[1] * rintf(dy / L32[1]);
                  dz -= L32[2] * rintf(dz / L32[2]);
                  if (dx * dx + dy * dy + dz * dz > reach * reach) continue;
                  if (ref_r2_scaled(m.x[i], m.y[i], m.z[i], m.x[j], m.y[j], m.z[j], len, sf) < 1.0) ov = true;
                }
              }
            }
          }
          if (ov) atomicOr(&v_ov, 1);
        }
      }
      __syncthreads();
      // decide, and rebuild the box (one thread)
      if (tid == 0 && !v_ov && v_u < vol_boltz(st->pressure, sb.vol, v_new, n, v_ratio)) {
        Box nbx = sb;
        if (vol_rebuild_box(st, n, v_new, margin, nbx)) {
          sb = nbx;
          v_acc = 1;
          vacc++;
        } else {
          atomicOr(&st->status, ST_BAD_CELL);
        }
      }
      __syncthreads();
      if (v_acc) {  // positions scaled and wrapped into the new box (src/moves.c:133-140)
        const double l0 = sb.len[0], l1 = sb.len[1], l2 = sb.len[2];
        for (int i = tid; i < n; i += nt) {
          m.x[i] = scale_wrap(m.x[i], sf, l0);
          m.y[i] = scale_wrap(m.y[i], sf, l1);
          m.z[i] = scale_wrap(m.z[i], sf, l2);
        }
      }
      __syncthreads();
    }
    if (sw == n_sweeps - 1 && tid == 0) {  // the last sweep's layout, as k_build leaves it
      st->params.sweep = s;
      for (int d = 0; d < 3; d++) st->params.shift32[d] = sh[d];
      for (int k = 0; k < 8; k++) st->params.perm[k] = perm_s[k];
    }
  }
  for (int i = tid; i < n; i += nt) {
    double *q = p.pos + 4 * (size_t)i;
    q[1] = m.x[i];
    q[2] = m.y[i];
    q[3] = m.z[i];
  }
  const unsigned long long a = warp_sum_u64(acc), o = warp_sum_u64(rej_o), bd = warp_sum_u64(rej_b);
  if ((tid & 31) == 0) {
    if (a) atomicAdd(&st->acc, a);
    if (o) atomicAdd(&st->rej_overlap, o);
    if (bd) atomicAdd(&st->rej_boundary, bd);
  }
  if (tid == 0) {
    st->sweep_base = s0 + (unsigned long long)n_sweeps;
    if (cavity) {
      st->cav_moves += cdone;
      st->cav_acc += cacc;
    }
    if (npt) {
      *p.box = sb;
      st->vol_moves += vmoves;
      st->vol_acc += vacc;
    }
  }
}

}  // namespace

size_t sweep_small_smem(int n, int ncell, int cap) {
  const int na = ncell / 8;  // active cells per pass (even counts per axis)
  if (n > 65535 || ncell > 65534 || na > kSmallThreads) return 0;
  // per particle: x, y, z, tx, ty, tz, id; per cell: count, offset; per
  // active cell: trial position, grid coordinates, particle, state, and the
  // draws of up to cap trials
  const size_t bytes = 38 * (size_t)n + 6 * (size_t)ncell + 39 * (size_t)na + 16 * (size_t)na * cap + 32;
  return bytes <= 224 * 1024 ? bytes : 0;  // of the 227 KB a block may have
}

// The shared-memory allowance is a property of the kernel, shared by every
// context on the device: it is set to the most the device allows beside the
// kernel's static shared memory, so that a context with a smaller system
// never lowers what an earlier, larger one needs.
template <bool CAV>
static bool allow_sweep_small(size_t smem) {
  int dev = 0, optin = 0;
  cudaFuncAttributes fa{};
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
      cudaFuncGetAttributes(&fa, k_sweep_small<CAV>) != cudaSuccess)
    return false;
  const int most = optin - (int)fa.sharedSizeBytes;
  return smem <= (size_t)most &&
         cudaFuncSetAttribute(k_sweep_small<CAV>, cudaFuncAttributeMaxDynamicSharedMemorySize, most) == cudaSuccess;
}

bool prepare_sweep_small(size_t smem) {
  if (smem == 0) return false;
  const bool ok = allow_sweep_small<false>(smem) && allow_sweep_small<true>(smem);
  if (!ok) cudaGetLastError();
  return ok;
}

void launch_sweep_small(const SysPtrs &p, int n_sweeps, bool npt, bool cavity, double margin, size_t smem,
                        cudaStream_t s) {
  if (cavity) k_sweep_small<true><<<1, kSmallThreads, smem, s>>>(p, n_sweeps, npt ? 1 : 0, margin);
  else k_sweep_small<false><<<1, kSmallThreads, smem, s>>>(p, n_sweeps, npt ? 1 : 0, margin);
}

}  // namespace hsmc
