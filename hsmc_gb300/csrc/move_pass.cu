// One colour pass of the checkerboard sweep (part_move / check_overlap,
// src/moves.c:27-80 and 157-212, for all cells of one colour at once).
//
// A group of G lanes owns one active cell at a time; consecutive groups take
// cells that are neighbours along x, so a warp's loads share cache lines.
// The 26 neighbour cells are split across the lanes and the lanes agree on
// each decision with one ballot.  Per cell, three rounds of memory traffic:
//   counts      of the cell and of the lane's neighbour cells, issued together;
//   slots       every slot of those cells copied with cp.async into shared
//               memory: the neighbours' into the group's pool (one column per
//               lane, so each lane screens an equal share), the cell's own
//               into the group's records; the lanes then add the periodic
//               image to the pool entries they copied;
//   positions   the FP64 coordinates of the cell's particles, by cp.async,
//               while the lanes rank the particles by id.
// Then n trials (n = particles in the cell), each on the particle of rank
// floor(u n) by id: FP64 proposal, confinement to the cell, single-precision
// screen four candidates at a time, FP64 re-evaluation of any pair within the
// guard band of contact.  Nothing per cell lives in local memory.
#include "engine.cuh"

namespace hsmc {

// Neighbour offsets of the 26 cells around a cell, packed (dx+1) | (dy+1)<<2
// | (dz+1)<<4, in the order x-major, the cell itself left out.
__constant__ unsigned char c_nbr[26] = {
    0x00, 0x10, 0x20, 0x04, 0x14, 0x24, 0x08, 0x18, 0x28, 0x01, 0x11, 0x21, 0x05,
    0x25, 0x09, 0x19, 0x29, 0x02, 0x12, 0x22, 0x06, 0x16, 0x26, 0x0a, 0x1a, 0x2a};

// Shared memory of one 128-thread block of k_move_pass<G, CAP>:
//   pool    PR x 128 float4: neighbour entry e of group gl sits in row e / G,
//           column gl * G + e % G (the column of lane e % G)
//   own_t   CAP x GPB float4: the cell's slots (grid coordinates, id)
//   own_x/y/z  CAP x GPB double: their FP64 coordinates
//   order   CAP x GPB byte: slot index of the particle of each id rank
template <int G, int CAP>
struct PassSmem {
  static constexpr int GPB = 128 / G;  // groups per block
  static constexpr int PC = 4 * CAP;   // pooled neighbour entries per group
  static constexpr int PR = PC / G;    // pool rows
  static constexpr size_t bytes =
      (size_t)PR * 128 * 16 + (size_t)CAP * GPB * 16 + (size_t)3 * CAP * GPB * 8 + (size_t)CAP * GPB;
  static constexpr size_t sm_bytes = 233472;  // shared memory of one SM
  static constexpr int by_smem = (int)(sm_bytes / (bytes + 1024));
  static constexpr int min_blocks = by_smem < 1 ? 1 : (by_smem > 8 ? 8 : by_smem);
};

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}

__device__ __forceinline__ void cp_async8(void *dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
               "l"(src)
               : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// Periodic image (a multiple of the box side) of neighbour `code` of cell
// (ix, iy, iz) as seen from that cell.
__device__ __forceinline__ void image_of(unsigned code, int ix, int iy, int iz, const int *nc, const float *L32,
                                         float &imx, float &imy, float &imz) {
  const int ox = (int)(code & 3u) - 1, oy = (int)((code >> 2) & 3u) - 1, oz = (int)(code >> 4) - 1;
  imx = (ix + ox < 0) ? -L32[0] : (ix + ox >= nc[0] ? L32[0] : 0.f);
  imy = (iy + oy < 0) ? -L32[1] : (iy + oy >= nc[1] ? L32[1] : 0.f);
  imz = (iz + oz < 0) ? -L32[2] : (iz + oz >= nc[2] ? L32[2] : 0.f);
}

__device__ __forceinline__ float dist2(float ux, float uy, float uz, const float4 &q) {
  const float dx = ux - q.x, dy = uy - q.y, dz = uz - q.z;
  return dx * dx + dy * dy + dz * dz;
}

template <int G, int CAP, bool TRACE, bool BATCH>
__global__ void __launch_bounds__(128, PassSmem<G, CAP>::min_blocks)
    k_move_pass(SysPtrs p1, const SysPtrs *reps, int pass) {
  // In a batch, blockIdx.y is the replica (see k_build).
  const SysPtrs p = BATCH ? reps[blockIdx.y] : p1;
  const uint32_t rep = BATCH ? blockIdx.y : 0u;
  static_assert(G == 1 || G == 2 || G == 4 || G == 8, "group size");
  using S = PassSmem<G, CAP>;
  constexpr int GPB = S::GPB, PC = S::PC, PR = S::PR;
  constexpr int NB = (26 + G - 1) / G;  // neighbour cells per lane
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4 *pool = reinterpret_cast<float4 *>(smem_raw);
  float4 *own_t = pool + PR * 128;
  double *own_x = reinterpret_cast<double *>(own_t + CAP * GPB);
  double *own_y = own_x + CAP * GPB;
  double *own_z = own_y + CAP * GPB;
  unsigned char *order = reinterpret_cast<unsigned char *>(own_z + CAP * GPB);

  const DevState *st = p.st;
  const Box *bx = p.box;
  const unsigned long long sweep = st->params.sweep;
  const int layout = (int)(sweep & 1ull);
  const int colour = st->params.perm[pass];
  const float sh[3] = {st->params.shift32[0], st->params.shift32[1], st->params.shift32[2]};
  const double dr = st->dr_max;
  const unsigned long long seed = st->seed;
  const unsigned long long seq = sweep * 8ull + (unsigned long long)pass;
  const double len[3] = {bx->len[0], bx->len[1], bx->len[2]};
  const double half[3] = {bx->half[0], bx->half[1], bx->half[2]};
  const float L32[3] = {bx->len32[0], bx->len32[1], bx->len32[2]};
  const float iw[3] = {bx->inv_w32[0], bx->inv_w32[1], bx->inv_w32[2]};
  const int nc[3] = {bx->nc[0], bx->nc[1], bx->nc[2]};
  const float band = bx->band;
  const float lo = 1.0f - band, hi = 1.0f + band;
  const int *__restrict__ cnt = cnt_of(p, layout);
  Slot *__restrict__ slot = slot_of(p, layout);
  double *__restrict__ pos = p.pos;

  // The first pass of a sweep clears the other layout for the next build.
  if (pass == 0) {
    int *other = cnt_of(p, layout ^ 1);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x) other[c] = 0;
  }

  const int tid = (int)threadIdx.x;
  const int lane = tid % G;
  const int gl = tid / G;  // group within the block
  const int col0 = tid - lane;
  const int group = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);
  const int groups = (int)((gridDim.x * blockDim.x) / G);
  const int gbase = (tid & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int hx = nc[0] >> 1, hy = nc[1] >> 1, hz = nc[2] >> 1;
  const int n_active = hx * hy * hz;
  const int cx = colour & 1, cy = (colour >> 1) & 1, cz = (colour >> 2) & 1;

  unsigned acc = 0, rej_o = 0, rej_b = 0, rechecks = 0;

  for (int ac = group; ac < n_active; ac += groups) {
    if (G > 1) __syncwarp(gmask);  // the previous cell's records are no longer read
    const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
    const int ix = 2 * ax + cx, iy = 2 * ay + cy, iz = 2 * az + cz;
    const int c = ix + nc[0] * (iy + nc[1] * iz);

    // (1) counts of the cell and of this lane's neighbour cells, issued
    // together.  An interior cell (most of them) reaches its neighbours by a
    // linear offset and sees no periodic image.
    const bool interior = ix > 0 && iy > 0 && iz > 0 && ix < nc[0] - 1 && iy < nc[1] - 1 && iz < nc[2] - 1;
    int nb_c[NB], nb_n[NB];
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const int o26 = lane + q * G;
      nb_c[q] = c;
      if (o26 < 26) {
        const unsigned code = c_nbr[o26];
        const int ox = (int)(code & 3u) - 1, oy = (int)((code >> 2) & 3u) - 1, oz = (int)(code >> 4) - 1;
        if (interior) {
          nb_c[q] = c + ox + nc[0] * (oy + nc[1] * oz);
        } else {
          int x = ix + ox, y = iy + oy, z = iz + oz;
          x += x < 0 ? nc[0] : (x >= nc[0] ? -nc[0] : 0);
          y += y < 0 ? nc[1] : (y >= nc[1] ? -nc[1] : 0);
          z += z < 0 ? nc[2] : (z >= nc[2] ? -nc[2] : 0);
          nb_c[q] = x + nc[0] * (y + nc[1] * z);
        }
      }
    }
    const int n = cnt[c];
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const int m = (lane + q * G < 26) ? cnt[nb_c[q]] : 0;
      nb_n[q] = m < CAP ? m : CAP;  // an overfull cell was flagged by the build
    }
    if (n == 0) continue;
    if (n > CAP) {
      if (lane == 0) atomicOr(&p.st->status, ST_CELL_OVERFLOW);
      continue;
    }

    // the group's neighbour entries: this lane's share starts at `first`
    int mine = 0;
#pragma unroll
    for (int q = 0; q < NB; q++) mine += nb_n[q];
    int incl = mine;
#pragma unroll
    for (int o = 1; o < G; o <<= 1) {
      const int v = __shfl_up_sync(gmask, incl, o, G);
      if (lane >= o) incl += v;
    }
    const int total = G > 1 ? __shfl_sync(gmask, incl, G - 1, G) : incl;
    const int first = incl - mine;
    const bool direct = total > PC;  // rare: screen straight from the slots

    // (2) slots, copied asynchronously into the pool and the records
    if (!direct) {
      int e = first;
#pragma unroll
      for (int q = 0; q < NB; q++) {
        const Slot *src = slot + (size_t)nb_c[q] * CAP;
        for (int k = 0; k < nb_n[q]; k++, e++) cp_async16(&pool[(e / G) * 128 + col0 + e % G], src + k);
      }
    }
    for (int j = lane; j < n; j += G) cp_async16(&own_t[j * GPB + gl], slot + (size_t)c * CAP + j);
    // the first trial's draws, computed while the copies are in flight
    U32x4 r_next = draw4(seed, rep << 8, (uint32_t)c, seq, TAG_MOVE);
    cp_async_wait_all();
    if (!direct && !interior) {  // periodic images of the entries this lane copied
      int e = first;
#pragma unroll
      for (int q = 0; q < NB; q++) {
        if (nb_n[q] == 0) continue;
        float imx, imy, imz;
        image_of(c_nbr[lane + q * G], ix, iy, iz, nc, L32, imx, imy, imz);
        if (imx != 0.f || imy != 0.f || imz != 0.f) {
          for (int k = 0; k < nb_n[q]; k++) {
            float4 &v = pool[((e + k) / G) * 128 + col0 + (e + k) % G];
            v.x = __fadd_rn(v.x, imx);
            v.y = __fadd_rn(v.y, imy);
            v.z = __fadd_rn(v.z, imz);
          }
        }
        e += nb_n[q];
      }
    }
    if (G > 1) __syncwarp(gmask);

    // (3) id ranks (the chain must not depend on the order the build's
    // atomics filled the slots) and the FP64 coordinates
    for (int j = lane; j < n; j += G) {
      const int id = __float_as_int(own_t[j * GPB + gl].w);
      int rank = 0;
      for (int k = 0; k < n; k++) rank += __float_as_int(own_t[k * GPB + gl].w) < id;
      order[rank * GPB + gl] = (unsigned char)j;
      const double *src = pos + 4 * (size_t)id;
      cp_async8(&own_x[j * GPB + gl], src + 1);
      cp_async8(&own_y[j * GPB + gl], src + 2);
      cp_async8(&own_z[j * GPB + gl], src + 3);
    }
    cp_async_wait_all();
    if (G > 1) __syncwarp(gmask);

    const int rows = (!direct && total > lane) ? (total - lane + G - 1) / G : 0;
    unsigned moved = 0;
    for (int trial = 0; trial < n; trial++) {
      const U32x4 r = r_next;
      if (trial + 1 < n) r_next = draw4(seed, (rep << 8) | (uint32_t)(trial + 1), (uint32_t)c, seq, TAG_MOVE);
      const int s = (int)__umulhi(r.x, (unsigned)n);  // rank of the moving particle
      const int js = order[s * GPB + gl] & (CAP - 1);  // a slot index below CAP
      const double nx = propose_axis(own_x[js * GPB + gl], centred_offset(r.y), dr, len[0]);
      const double ny = propose_axis(own_y[js * GPB + gl], centred_offset(r.z), dr, len[1]);
      const double nz = propose_axis(own_z[js * GPB + gl], centred_offset(r.w), dr, len[2]);
      int c0, c1, c2;
      float ux, uy, uz;
      axis_cell(__double2float_rn(nx), sh[0], L32[0], iw[0], nc[0], c0, ux);
      axis_cell(__double2float_rn(ny), sh[1], L32[1], iw[1], nc[1], c1, uy);
      axis_cell(__double2float_rn(nz), sh[2], L32[2], iw[2], nc[2], c2, uz);
      const unsigned rc_before = rechecks;
      int decision;
      if (c0 != ix || c1 != iy || c2 != iz) {
        decision = 2;  // the move would leave the active cell
      } else {
        bool ov = false;
        // the rest of the cell
        for (int k = lane; k < n && !ov; k += G) {
          if (k == js) continue;
          const float r2 = dist2(ux, uy, uz, own_t[k * GPB + gl]);
          if (r2 < lo) {
            ov = true;
          } else if (r2 <= hi) {
            rechecks++;
            ov = ref_r2(nx, ny, nz, own_x[k * GPB + gl], own_y[k * GPB + gl], own_z[k * GPB + gl], len, half) < 1.0;
          }
        }
        if (!direct) {
          const float4 *mine_col = pool + tid;
          int w = 0;
          for (; w + 4 <= rows && !ov; w += 4) {
            const float4 a0 = mine_col[w * 128], a1 = mine_col[(w + 1) * 128];
            const float4 a2 = mine_col[(w + 2) * 128], a3 = mine_col[(w + 3) * 128];
            const float r0 = dist2(ux, uy, uz, a0), r1 = dist2(ux, uy, uz, a1);
            const float r2 = dist2(ux, uy, uz, a2), r3 = dist2(ux, uy, uz, a3);
            if (fminf(fminf(r0, r1), fminf(r2, r3)) <= hi) {
              const float rr[4] = {r0, r1, r2, r3};
              const int ids[4] = {__float_as_int(a0.w), __float_as_int(a1.w), __float_as_int(a2.w),
                                  __float_as_int(a3.w)};
#pragma unroll
              for (int u = 0; u < 4; u++) {
                if (ov) break;
                if (rr[u] < lo) {
                  ov = true;
                } else if (rr[u] <= hi) {
                  rechecks++;
                  double ox, oy, oz;
                  load_xyz(pos, ids[u], ox, oy, oz);
                  ov = ref_r2(nx, ny, nz, ox, oy, oz, len, half) < 1.0;
                }
              }
            }
          }
          for (; w < rows && !ov; w++) {
            const float4 a = mine_col[w * 128];
            const float r2 = dist2(ux, uy, uz, a);
            if (r2 < lo) {
              ov = true;
            } else if (r2 <= hi) {
              rechecks++;
              double ox, oy, oz;
              load_xyz(pos, __float_as_int(a.w), ox, oy, oz);
              ov = ref_r2(nx, ny, nz, ox, oy, oz, len, half) < 1.0;
            }
          }
        } else {
#pragma unroll
          for (int q = 0; q < NB; q++) {
            if (nb_n[q] == 0) continue;
            float imx, imy, imz;
            image_of(c_nbr[lane + q * G], ix, iy, iz, nc, L32, imx, imy, imz);
            for (int k = 0; k < nb_n[q] && !ov; k++) {
              const Slot o = slot[(size_t)nb_c[q] * CAP + k];
              const float4 a = make_float4(__fadd_rn(o.x, imx), __fadd_rn(o.y, imy), __fadd_rn(o.z, imz), 0.f);
              const float r2 = dist2(ux, uy, uz, a);
              if (r2 < lo) {
                ov = true;
              } else if (r2 <= hi) {
                rechecks++;
                double px, py, pz;
                load_xyz(pos, o.id, px, py, pz);
                ov = ref_r2(nx, ny, nz, px, py, pz, len, half) < 1.0;
              }
            }
          }
        }
        if (G > 1) ov = __ballot_sync(gmask, ov) != 0u;
        decision = ov ? 1 : 0;
      }
      const int moving_id = __float_as_int(own_t[js * GPB + gl].w);
      if (decision == 0) {
        if (G > 1) __syncwarp(gmask);  // every lane has read this trial's records
        if (lane == 0) {
          own_x[js * GPB + gl] = nx;
          own_y[js * GPB + gl] = ny;
          own_z[js * GPB + gl] = nz;
          own_t[js * GPB + gl] = make_float4(ux, uy, uz, __int_as_float(moving_id));
        }
        moved |= 1u << js;
        if (G > 1) __syncwarp(gmask);
      }
      if (lane == 0) {
        acc += decision == 0;
        rej_o += decision == 1;
        rej_b += decision == 2;
      }
      if (TRACE) {
        bool any_rc = rechecks != rc_before;
        if (G > 1) any_rc = __ballot_sync(gmask, any_rc) != 0u;
        if (lane == 0) {
          const unsigned long long at = atomicAdd(&p.st->trace_count, 1ull);
          if (at < p.trace_cap) {
            uint32_t *rec = p.trace + 12 * at;
            rec[0] = (uint32_t)seq;
            rec[1] = (uint32_t)c;
            rec[2] = (uint32_t)trial;
            rec[3] = (uint32_t)moving_id;
            rec[4] = r.y;
            rec[5] = r.z;
            rec[6] = r.w;
            rec[7] = (uint32_t)decision;
            rec[8] = __float_as_uint(sh[0]);
            rec[9] = __float_as_uint(sh[1]);
            rec[10] = __float_as_uint(sh[2]);
            rec[11] = any_rc ? 1u : 0u;
          } else {
            atomicOr(&p.st->status, ST_TRACE_FULL);
          }
        }
      }
    }
    for (int j = lane; j < n; j += G) {
      if (!((moved >> j) & 1u)) continue;
      const float4 t = own_t[j * GPB + gl];
      double *pp = pos + 4 * (size_t)__float_as_int(t.w);
      pp[1] = own_x[j * GPB + gl];
      pp[2] = own_y[j * GPB + gl];
      pp[3] = own_z[j * GPB + gl];
      slot[(size_t)c * CAP + j] = Slot{t.x, t.y, t.z, __float_as_int(t.w)};
    }
  }

  const unsigned long long a64 = warp_sum_u64(acc), o64 = warp_sum_u64(rej_o), b64 = warp_sum_u64(rej_b),
                           r64 = warp_sum_u64(rechecks);
  if ((threadIdx.x & 31) == 0) {
    DevState *ws = p.st;
    if (a64) atomicAdd(&ws->acc, a64);
    if (o64) atomicAdd(&ws->rej_overlap, o64);
    if (b64) atomicAdd(&ws->rej_boundary, b64);
    if (r64) atomicAdd(&ws->rechecks, r64);
  }
}

// ------------------------------------------------------------------ launch
template <int G, int CAP>
static size_t pass_smem() {
  return PassSmem<G, CAP>::bytes;
}

static int smem_optin_limit() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

// Dynamic shared memory above 48 KB has to be allowed per kernel and device,
// before any launch is captured into a graph: prepare_move_pass does it for
// every variant that fits on the current device.
template <int G, int CAP, bool TRACE, bool BATCH>
static void allow_smem() {
  if (pass_smem<G, CAP>() > (size_t)smem_optin_limit()) return;
  cudaFuncSetAttribute(k_move_pass<G, CAP, TRACE, BATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)pass_smem<G, CAP>());
}

template <int G, int CAP>
static void allow_all() {
  allow_smem<G, CAP, false, false>();
  allow_smem<G, CAP, true, false>();
  allow_smem<G, CAP, false, true>();
}

template <int G>
static void allow_caps() {
  allow_all<G, 8>();
  allow_all<G, 16>();
  allow_all<G, 32>();
}

void prepare_move_pass() {
  allow_caps<1>();
  allow_caps<2>();
  allow_caps<4>();
  allow_caps<8>();
}

static size_t smem_for(int group, int cap) {
  const int c = cap <= 8 ? 8 : (cap <= 16 ? 16 : 32);
  // bytes grow as cap / group (PassSmem): evaluate the cap = 8 layout and scale
  return PassSmem<1, 8>::bytes * (size_t)(c / 8) / (size_t)group;
}

bool move_pass_fits(int group, int cap) {
  if (group != 1 && group != 2 && group != 4 && group != 8) return false;
  return smem_for(group, cap) <= (size_t)smem_optin_limit();
}

// Groups per pass = active cells (an eighth of the grid); one wave when the
// occupancy allows it, grid-stride otherwise.
template <int G, int CAP>
static int pass_blocks_for(int ncell_alloc, int num_sms) {
  if (pass_smem<G, CAP>() > (size_t)smem_optin_limit()) return 0;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_move_pass<G, CAP, false, false>, 128,
                                                pass_smem<G, CAP>());
  if (per_sm < 1) per_sm = 1;
  const long long threads = (long long)(ncell_alloc / 8) * G;
  const int need = (int)((threads + 127) / 128);
  const int cap = per_sm * num_sms;
  return need < cap ? (need > 0 ? need : 1) : cap;
}

template <int G>
static int pass_blocks_g(int cap, int ncell_alloc, int num_sms) {
  switch (cap) {
    case 8: return pass_blocks_for<G, 8>(ncell_alloc, num_sms);
    case 16: return pass_blocks_for<G, 16>(ncell_alloc, num_sms);
    default: return pass_blocks_for<G, 32>(ncell_alloc, num_sms);
  }
}

int move_pass_grid(int group, int cap, int ncell_alloc, int num_sms) {
  switch (group) {
    case 1: return pass_blocks_g<1>(cap, ncell_alloc, num_sms);
    case 2: return pass_blocks_g<2>(cap, ncell_alloc, num_sms);
    case 4: return pass_blocks_g<4>(cap, ncell_alloc, num_sms);
    default: return pass_blocks_g<8>(cap, ncell_alloc, num_sms);
  }
}

template <int G, int CAP>
static void launch_gc(const SysPtrs &p, int pass, bool trace, int grid, cudaStream_t s) {
  const size_t sm = pass_smem<G, CAP>();
  if (trace) k_move_pass<G, CAP, true, false><<<grid, 128, sm, s>>>(p, nullptr, pass);
  else k_move_pass<G, CAP, false, false><<<grid, 128, sm, s>>>(p, nullptr, pass);
}

template <int G, int CAP>
static void launch_batch_gc(const SysPtrs *reps, int n_reps, int pass, int grid_x, cudaStream_t s) {
  k_move_pass<G, CAP, false, true>
      <<<dim3((unsigned)grid_x, (unsigned)n_reps), 128, pass_smem<G, CAP>(), s>>>(SysPtrs{}, reps, pass);
}

// Blocks per replica for the batched pass: enough groups for the largest
// replica's active cells; groups past a smaller replica's cells exit at once.
int move_pass_grid_batch(int group, int max_ncell) {
  const long long threads = (long long)(max_ncell / 8) * group;
  const int x = (int)((threads + 127) / 128);
  return x > 0 ? x : 1;
}

void launch_move_pass_batch(const SysPtrs *reps, int n_reps, int cap, int pass, int group, int grid_x,
                            cudaStream_t s) {
#define HSMC_BATCH_CAP(G)                                                      \
  switch (cap) {                                                               \
    case 8: launch_batch_gc<G, 8>(reps, n_reps, pass, grid_x, s); break;       \
    case 16: launch_batch_gc<G, 16>(reps, n_reps, pass, grid_x, s); break;     \
    default: launch_batch_gc<G, 32>(reps, n_reps, pass, grid_x, s); break;     \
  }
  switch (group) {
    case 1: HSMC_BATCH_CAP(1) break;
    case 2: HSMC_BATCH_CAP(2) break;
    case 4: HSMC_BATCH_CAP(4) break;
    default: HSMC_BATCH_CAP(8) break;
  }
#undef HSMC_BATCH_CAP
}

template <int G>
static void launch_g(const SysPtrs &p, int pass, bool trace, int grid, cudaStream_t s) {
  switch (p.cap) {
    case 8: launch_gc<G, 8>(p, pass, trace, grid, s); break;
    case 16: launch_gc<G, 16>(p, pass, trace, grid, s); break;
    default: launch_gc<G, 32>(p, pass, trace, grid, s); break;
  }
}

void launch_move_pass(const SysPtrs &p, int pass, int group, bool trace, int grid, cudaStream_t s) {
  switch (group) {
    case 1: launch_g<1>(p, pass, trace, grid, s); break;
    case 2: launch_g<2>(p, pass, trace, grid, s); break;
    case 4: launch_g<4>(p, pass, trace, grid, s); break;
    default: launch_g<8>(p, pass, trace, grid, s); break;
  }
}

}  // namespace hsmc
