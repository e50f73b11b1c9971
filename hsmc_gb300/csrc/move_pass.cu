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
// floor(u n) by id: FP64 proposal (its axes shared out over the group's
// lanes), confinement to the cell, single-precision screen four candidates at
// a time, FP64 re-evaluation of any pair within the guard band of contact.
// Each pass is a programmatic dependent launch of the one before.  Nothing per
// cell lives in local memory.
#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "screen.cuh"

namespace cg = cooperative_groups;

namespace hsmc {

// Shared memory of one 128-thread block of k_move_pass<G, CAP>:
//   pool    PR x 128 float4: neighbour entry e of group gl sits in row e / G,
//           column gl * G + e % G (the column of lane e % G)
//   own_t   CAP x GPB float4: the cell's slots (grid coordinates, id)
//   own_x/y/z  CAP x GPB double: their FP64 coordinates
//   order   CAP x GPB byte: slot index of the particle of each id rank
// The pool holds 4 CAP neighbour entries per group, plus one row (G more)
// where that costs no resident block.  A cell whose neighbours hold more
// than PC particles is screened straight from global memory, which is many
// times slower and makes its warp the last of the pass: at 0.89 particles
// per cell (rho = 0.85) 26 neighbour cells hold 23 on average, and more than
// 32 about once per 30,000 occupied cells, more than 34 far more rarely.
template <int G, int CAP>
struct PassSmem {
  static constexpr int GPB = 128 / G;         // groups per block
  static constexpr size_t sm_bytes = 233472;  // shared memory of one SM
  static constexpr size_t fixed = (size_t)CAP * GPB * 16 + (size_t)3 * CAP * GPB * 8 + (size_t)CAP * GPB;
  static constexpr int fit(int rows) {
    const int b = (int)(sm_bytes / ((size_t)rows * 128 * 16 + fixed + 1024));
    return b < 1 ? 1 : (b > 8 ? 8 : b);
  }
  static constexpr int PR = fit(4 * CAP / G + 1) == fit(4 * CAP / G) ? 4 * CAP / G + 1 : 4 * CAP / G;  // pool rows
  static constexpr int PC = PR * G;  // pooled neighbour entries per group
  static constexpr size_t bytes = (size_t)PR * 128 * 16 + fixed;
  static constexpr int min_blocks = fit(PR);
};

// The slot copies bypass L1 (.cg): allocating them there measured 10 % slower
// per sweep (the slot lines are read once per pass, and the L1 is better
// left to the counts, whose lines neighbouring cells share).
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"((unsigned)__cvta_generic_to_shared(dst)),
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

// Everything a pass needs that is fixed for the launch (or the pass).
struct PassEnv {
  const int *cnt;
  Slot *slot;
  double *pos;
  DevState *st;
  double dr;
  unsigned long long seed, seq;
  double len[3], half[3];
  float L32[3], iw[3], sh[3];
  int nc[3];
  float lo, hi;
  int frozen;  // particles below this id stay in place (the cavities of a cavity run)
  uint32_t rep;
  uint32_t *trace;
  unsigned long long trace_cap;
};

struct PassSm {
  float4 *pool, *own_t;
  double *own_x, *own_y, *own_z;
  unsigned char *order;
};

struct PassTally {
  unsigned acc = 0, rej_o = 0, rej_b = 0, rechecks = 0;
};

// Loads of data that other blocks of the same launch write (the dataflow
// schedule) must bypass the non-coherent L1: CG selects the L2-only forms.
// (Slot copies are L2-only in every schedule, see cp_async16.)
template <bool CG>
__device__ __forceinline__ void copy16(void *dst, const void *src) {
  cp_async16(dst, src);
}

template <bool CG>
__device__ __forceinline__ void xyz_of(const double *pos, int id, double &x, double &y, double &z) {
  if (CG) {
    const double2 a = __ldcg(reinterpret_cast<const double2 *>(pos + 4 * (size_t)id));
    const double2 b = __ldcg(reinterpret_cast<const double2 *>(pos + 4 * (size_t)id + 2));
    x = a.y;
    y = b.x;
    z = b.y;
  } else {
    load_xyz(pos, id, x, y, z);
  }
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release(uint32_t *p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

// The n trial moves of one active cell (ix, iy, iz) by one group of G lanes.
// FLOW: other blocks of the launch write the data, so read through L2 only.
template <int G, int CAP, bool TRACE, bool FLOW>
__device__ __forceinline__ void move_cell(const PassEnv &e, const PassSm &m, int tid, int lane, int gl, int col0,
                                          unsigned gmask, int ix, int iy, int iz, PassTally &t) {
  constexpr int GPB = PassSmem<G, CAP>::GPB, PC = PassSmem<G, CAP>::PC;
  constexpr int NB = (26 + G - 1) / G;  // neighbour cells per lane
  const int *nc = e.nc;
  const int c = ix + nc[0] * (iy + nc[1] * iz);

  // (1) counts of the cell and of this lane's neighbour cells, issued
  // together.  An interior cell (most of them) reaches its neighbours by a
  // linear offset and sees no periodic image.
  const bool interior = ix > 0 && iy > 0 && iz > 0 && ix < nc[0] - 1 && iy < nc[1] - 1 && iz < nc[2] - 1;
  int nb_c[NB], nb_n[NB];
#pragma unroll
  for (int q = 0; q < NB; q++) {
    const int o26 = lane + q * G;
    nb_c[q] = o26 < 26 ? neighbour_cell(c_nbr[o26], ix, iy, iz, c, nc, interior) : c;
  }
  const int n = e.cnt[c];
#pragma unroll
  for (int q = 0; q < NB; q++) {
    const int mm = (lane + q * G < 26) ? e.cnt[nb_c[q]] : 0;
    nb_n[q] = mm < CAP ? mm : CAP;  // an overfull cell was flagged by the build
  }
  if (n == 0) return;
  if (n > CAP) {
    if (lane == 0) atomicOr(&e.st->status, ST_CELL_OVERFLOW);
    return;
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
    int k0 = first;
#pragma unroll
    for (int q = 0; q < NB; q++) {
      const Slot *src = e.slot + (size_t)nb_c[q] * CAP;
      for (int k = 0; k < nb_n[q]; k++, k0++) copy16<FLOW>(&m.pool[(k0 / G) * 128 + col0 + k0 % G], src + k);
    }
  }
  for (int j = lane; j < n; j += G) copy16<FLOW>(&m.own_t[j * GPB + gl], e.slot + (size_t)c * CAP + j);
  // the first trial's draws, computed while the copies are in flight
  U32x4 r_next = draw4(e.seed, e.rep << 8, (uint32_t)c, e.seq, TAG_MOVE);
  cp_async_wait_all();
  if (!direct && !interior) {  // periodic images of the entries this lane copied
    int k0 = first;
#pragma unroll
    for (int q = 0; q < NB; q++) {
      if (nb_n[q] == 0) continue;
      float imx, imy, imz;
      image_of(c_nbr[lane + q * G], ix, iy, iz, nc, e.L32, imx, imy, imz);
      if (imx != 0.f || imy != 0.f || imz != 0.f) {
        for (int k = 0; k < nb_n[q]; k++) {
          float4 &v = m.pool[((k0 + k) / G) * 128 + col0 + (k0 + k) % G];
          v.x = __fadd_rn(v.x, imx);
          v.y = __fadd_rn(v.y, imy);
          v.z = __fadd_rn(v.z, imz);
        }
      }
      k0 += nb_n[q];
    }
  }
  if (G > 1) __syncwarp(gmask);

  // (3) id ranks (the chain must not depend on the order the build's
  // atomics filled the slots) and the FP64 coordinates
  for (int j = lane; j < n; j += G) {
    const int id = __float_as_int(m.own_t[j * GPB + gl].w);
    int rank = 0;
    for (int k = 0; k < n; k++) rank += __float_as_int(m.own_t[k * GPB + gl].w) < id;
    m.order[rank * GPB + gl] = (unsigned char)j;
    if (FLOW) {
      double x, y, z;
      xyz_of<true>(e.pos, id, x, y, z);
      m.own_x[j * GPB + gl] = x;
      m.own_y[j * GPB + gl] = y;
      m.own_z[j * GPB + gl] = z;
    } else {
      const double *src = e.pos + 4 * (size_t)id;
      cp_async8(&m.own_x[j * GPB + gl], src + 1);
      cp_async8(&m.own_y[j * GPB + gl], src + 2);
      cp_async8(&m.own_z[j * GPB + gl], src + 3);
    }
  }
  if (!FLOW) cp_async_wait_all();
  if (G > 1) __syncwarp(gmask);

  // This lane's column holds `rows` entries; it is padded with far-away
  // entries (never within the band of contact, never rechecked) up to a
  // multiple of four rows where the pool has room, so the screen runs four
  // candidates at a time without a serial remainder.
  int rows = (!direct && total > lane) ? (total - lane + G - 1) / G : 0;
  {
    constexpr int PR = PassSmem<G, CAP>::PR;
    const int rows4 = (rows + 3) & ~3;
    if (rows4 <= PR) {
      for (int w = rows; w < rows4; w++) m.pool[w * 128 + tid] = make_float4(1e30f, 1e30f, 1e30f, __int_as_float(-1));
      rows = rows4;
    }
  }
  const float lo = e.lo, hi = e.hi;
  unsigned moved = 0;
  for (int trial = 0; trial < n; trial++) {
    const U32x4 r = r_next;
    if (trial + 1 < n) r_next = draw4(e.seed, (e.rep << 8) | (uint32_t)(trial + 1), (uint32_t)c, e.seq, TAG_MOVE);
    const int s = (int)__umulhi(r.x, (unsigned)n);          // rank of the moving particle
    const int js = m.order[s * GPB + gl] & (CAP - 1);        // a slot index below CAP
    double nx, ny, nz;
    int c0, c1, c2;
    float ux, uy, uz;
    if (G >= 4) {
      // Lanes 0, 1 and 2 of each quad move x, y and z (lane 3 repeats z) in
      // one round of the FP64 pipe, then every lane reads the three.
      const int ax = (lane & 3) > 2 ? 2 : (lane & 3);
      const double la = ax == 0 ? e.len[0] : (ax == 1 ? e.len[1] : e.len[2]);
      const double xa = ax == 0 ? m.own_x[js * GPB + gl] : (ax == 1 ? m.own_y[js * GPB + gl] : m.own_z[js * GPB + gl]);
      double va = __dadd_rn(xa, __dmul_rn(centred_offset(ax == 0 ? r.y : (ax == 1 ? r.z : r.w)), e.dr));
      const bool oa = gt_pos(va, la);
      const bool wa = oa || lt_zero(va);
      if (__any_sync(gmask, wa)) {
        if (wa) va = __dadd_rn(va, oa ? -la : la);
      }
      int ca;
      float ua;
      axis_cell(__double2float_rn(va), ax == 0 ? e.sh[0] : (ax == 1 ? e.sh[1] : e.sh[2]),
                ax == 0 ? e.L32[0] : (ax == 1 ? e.L32[1] : e.L32[2]), ax == 0 ? e.iw[0] : (ax == 1 ? e.iw[1] : e.iw[2]),
                ax == 0 ? nc[0] : (ax == 1 ? nc[1] : nc[2]), ca, ua);
      nx = __shfl_sync(gmask, va, 0, 4);
      ny = __shfl_sync(gmask, va, 1, 4);
      nz = __shfl_sync(gmask, va, 2, 4);
      ux = __shfl_sync(gmask, ua, 0, 4);
      uy = __shfl_sync(gmask, ua, 1, 4);
      uz = __shfl_sync(gmask, ua, 2, 4);
      c0 = __shfl_sync(gmask, ca, 0, 4);
      c1 = __shfl_sync(gmask, ca, 1, 4);
      c2 = __shfl_sync(gmask, ca, 2, 4);
    } else if (G >= 2) {
      // The FP64 work of the proposal is shared by the group's lanes: lane 0
      // moves x, lane 1 y, both z, and they swap x and y.  The narrow FP64 pipe
      // costs a warp instruction whatever the lanes it serves, and every warp
      // of an SM reaches this point at about the same time, so this cuts the
      // queue there by a third.  The periodic wrap is one add of -L or +L
      // (v - L and v + (-L) are the same IEEE operation), issued only when a
      // lane's proposal left the box.
      const int a = lane & 1;
      const double la = a ? e.len[1] : e.len[0];
      double va = __dadd_rn(a ? m.own_y[js * GPB + gl] : m.own_x[js * GPB + gl],
                            __dmul_rn(centred_offset(a ? r.z : r.y), e.dr));
      double vz = __dadd_rn(m.own_z[js * GPB + gl], __dmul_rn(centred_offset(r.w), e.dr));
      const bool oa = gt_pos(va, la), oz = gt_pos(vz, e.len[2]);
      const bool wa = oa || lt_zero(va), wz = oz || lt_zero(vz);
      if (__any_sync(gmask, wa || wz)) {
        if (wa) va = __dadd_rn(va, oa ? -la : la);
        if (wz) vz = __dadd_rn(vz, oz ? -e.len[2] : e.len[2]);
      }
      int ca;
      float ua;
      axis_cell(__double2float_rn(va), a ? e.sh[1] : e.sh[0], a ? e.L32[1] : e.L32[0], a ? e.iw[1] : e.iw[0],
                a ? nc[1] : nc[0], ca, ua);
      axis_cell(__double2float_rn(vz), e.sh[2], e.L32[2], e.iw[2], nc[2], c2, uz);
      const double vb = __shfl_xor_sync(gmask, va, 1);
      const float ub = __shfl_xor_sync(gmask, ua, 1);
      const int cb = __shfl_xor_sync(gmask, ca, 1);
      nx = a ? vb : va;
      ny = a ? va : vb;
      nz = vz;
      ux = a ? ub : ua;
      uy = a ? ua : ub;
      c0 = a ? cb : ca;
      c1 = a ? ca : cb;
    } else {
      nx = propose_axis(m.own_x[js * GPB + gl], centred_offset(r.y), e.dr, e.len[0]);
      ny = propose_axis(m.own_y[js * GPB + gl], centred_offset(r.z), e.dr, e.len[1]);
      nz = propose_axis(m.own_z[js * GPB + gl], centred_offset(r.w), e.dr, e.len[2]);
      axis_cell(__double2float_rn(nx), e.sh[0], e.L32[0], e.iw[0], nc[0], c0, ux);
      axis_cell(__double2float_rn(ny), e.sh[1], e.L32[1], e.iw[1], nc[1], c1, uy);
      axis_cell(__double2float_rn(nz), e.sh[2], e.L32[2], e.iw[2], nc[2], c2, uz);
    }
    const unsigned rc_before = t.rechecks;
    const int moving_id = __float_as_int(m.own_t[js * GPB + gl].w);
    int decision;
    if (moving_id < e.frozen) {
      decision = 4;  // a cavity: moved by the cavity stage, not here
    } else if (c0 != ix || c1 != iy || c2 != iz) {
      decision = 2;  // the move would leave the active cell
    } else {
      bool ov = false;
      // the rest of the cell
      for (int k = lane; k < n && !ov; k += G) {
        if (k == js) continue;
        const float r2 = dist2(ux, uy, uz, m.own_t[k * GPB + gl]);
        if (r2 < lo) {
          ov = true;
        } else if (r2 <= hi) {
          t.rechecks++;
          ov = ref_r2(nx, ny, nz, m.own_x[k * GPB + gl], m.own_y[k * GPB + gl], m.own_z[k * GPB + gl], e.len,
                      e.half) < 1.0;
        }
      }
      if (!direct) {
        const float4 *col = m.pool + tid;
        int w = 0;
        for (; w + 4 <= rows && !ov; w += 4) {
          const float4 a0 = col[w * 128], a1 = col[(w + 1) * 128];
          const float4 a2 = col[(w + 2) * 128], a3 = col[(w + 3) * 128];
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
                t.rechecks++;
                double ox, oy, oz;
                xyz_of<FLOW>(e.pos, ids[u], ox, oy, oz);
                ov = ref_r2(nx, ny, nz, ox, oy, oz, e.len, e.half) < 1.0;
              }
            }
          }
        }
        for (; w < rows && !ov; w++) {
          const float4 a = col[w * 128];
          const float r2 = dist2(ux, uy, uz, a);
          if (r2 < lo) {
            ov = true;
          } else if (r2 <= hi) {
            t.rechecks++;
            double ox, oy, oz;
            xyz_of<FLOW>(e.pos, __float_as_int(a.w), ox, oy, oz);
            ov = ref_r2(nx, ny, nz, ox, oy, oz, e.len, e.half) < 1.0;
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < NB; q++) {
          // recomputed here so the staging arrays need not live through the trials
          const int o26 = lane + q * G;
          if (o26 >= 26) continue;
          const unsigned code = c_nbr[o26];
          const int nbc = neighbour_cell(code, ix, iy, iz, c, nc, interior);
          const int mm = e.cnt[nbc];
          const int nbn = mm < CAP ? mm : CAP;
          if (nbn == 0) continue;
          float imx, imy, imz;
          image_of(code, ix, iy, iz, nc, e.L32, imx, imy, imz);
          for (int k = 0; k < nbn && !ov; k++) {
            const Slot *sp = e.slot + (size_t)nbc * CAP + k;
            Slot o;
            if (FLOW) {
              const float4 v = __ldcg(reinterpret_cast<const float4 *>(sp));
              o = Slot{v.x, v.y, v.z, __float_as_int(v.w)};
            } else {
              o = *sp;
            }
            const float4 a = make_float4(__fadd_rn(o.x, imx), __fadd_rn(o.y, imy), __fadd_rn(o.z, imz), 0.f);
            const float r2 = dist2(ux, uy, uz, a);
            if (r2 < lo) {
              ov = true;
            } else if (r2 <= hi) {
              t.rechecks++;
              double px, py, pz;
              xyz_of<FLOW>(e.pos, o.id, px, py, pz);
              ov = ref_r2(nx, ny, nz, px, py, pz, e.len, e.half) < 1.0;
            }
          }
        }
      }
      if (G > 1) ov = __ballot_sync(gmask, ov) != 0u;
      decision = ov ? 1 : 0;
    }
    if (decision == 0) {
      if (G > 1) __syncwarp(gmask);  // every lane has read this trial's records
      if (lane == 0) {
        m.own_x[js * GPB + gl] = nx;
        m.own_y[js * GPB + gl] = ny;
        m.own_z[js * GPB + gl] = nz;
        m.own_t[js * GPB + gl] = make_float4(ux, uy, uz, __int_as_float(moving_id));
      }
      moved |= 1u << js;
      if (G > 1) __syncwarp(gmask);
    }
    if (lane == 0) {
      t.acc += decision == 0;
      t.rej_o += decision == 1;
      t.rej_b += decision == 2;
    }
    if (TRACE) {
      bool any_rc = t.rechecks != rc_before;
      if (G > 1) any_rc = __ballot_sync(gmask, any_rc) != 0u;
      if (lane == 0) {
        const unsigned long long at = atomicAdd(&e.st->trace_count, 1ull);
        if (at < e.trace_cap) {
          uint32_t *rec = e.trace + 12 * at;
          rec[0] = (uint32_t)e.seq;
          rec[1] = (uint32_t)c;
          rec[2] = (uint32_t)trial;
          rec[3] = (uint32_t)moving_id;
          rec[4] = r.y;
          rec[5] = r.z;
          rec[6] = r.w;
          rec[7] = (uint32_t)decision;
          rec[8] = __float_as_uint(e.sh[0]);
          rec[9] = __float_as_uint(e.sh[1]);
          rec[10] = __float_as_uint(e.sh[2]);
          rec[11] = any_rc ? 1u : 0u;
        } else {
          atomicOr(&e.st->status, ST_TRACE_FULL);
        }
      }
    }
  }
  for (int j = lane; j < n; j += G) {
    if (!((moved >> j) & 1u)) continue;
    const float4 tt = m.own_t[j * GPB + gl];
    double *pp = e.pos + 4 * (size_t)__float_as_int(tt.w);
    pp[1] = m.own_x[j * GPB + gl];
    pp[2] = m.own_y[j * GPB + gl];
    pp[3] = m.own_z[j * GPB + gl];
    e.slot[(size_t)c * CAP + j] = Slot{tt.x, tt.y, tt.z, __float_as_int(tt.w)};
  }
}

template <int G, int CAP>
__device__ __forceinline__ PassSm pass_smem_ptrs(unsigned char *raw) {
  constexpr int GPB = PassSmem<G, CAP>::GPB, PR = PassSmem<G, CAP>::PR;
  PassSm m;
  m.pool = reinterpret_cast<float4 *>(raw);
  m.own_t = m.pool + PR * 128;
  m.own_x = reinterpret_cast<double *>(m.own_t + CAP * GPB);
  m.own_y = m.own_x + CAP * GPB;
  m.own_z = m.own_y + CAP * GPB;
  m.order = reinterpret_cast<unsigned char *>(m.own_z + CAP * GPB);
  return m;
}

__device__ __forceinline__ PassEnv pass_env(const SysPtrs &p, uint32_t rep, int layout) {
  PassEnv e;
  const DevState *st = p.st;
  const Box *bx = p.box;
  e.cnt = cnt_of(p, layout);
  e.slot = slot_of(p, layout);
  e.pos = p.pos;
  e.st = p.st;
  e.dr = st->dr_max;
  e.seed = st->seed;
  e.seq = 0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    e.len[d] = bx->len[d];
    e.half[d] = bx->half[d];
    e.L32[d] = bx->len32[d];
    e.iw[d] = bx->inv_w32[d];
    e.sh[d] = st->params.shift32[d];
    e.nc[d] = bx->nc[d];
  }
  e.lo = 1.0f - bx->band;
  e.hi = 1.0f + bx->band;
  e.frozen = st->frozen;
  e.rep = rep;
  e.trace = p.trace;
  e.trace_cap = p.trace_cap;
  return e;
}

__device__ __forceinline__ void add_tally(const PassTally &t, DevState *ws) {
  const unsigned long long a64 = warp_sum_u64(t.acc), o64 = warp_sum_u64(t.rej_o), b64 = warp_sum_u64(t.rej_b),
                           r64 = warp_sum_u64(t.rechecks);
  if ((threadIdx.x & 31) == 0) {
    if (a64) atomicAdd(&ws->acc, a64);
    if (o64) atomicAdd(&ws->rej_overlap, o64);
    if (b64) atomicAdd(&ws->rej_boundary, b64);
    if (r64) atomicAdd(&ws->rechecks, r64);
  }
}

// One colour pass: every active cell of the colour, then a kernel boundary.
// In a batch (BATCH) the grid covers the active cells of every replica of
// one cell capacity (gstart: their prefix sums); each group finds its
// replica, whose batch index (rep_ids) enters the random counters, and the
// counters are summed per replica.  Given the pooled count arrays, the first
// pass also clears their other layout.
template <int G, int CAP, bool TRACE, bool BATCH>
__global__ void __launch_bounds__(128, PassSmem<G, CAP>::min_blocks)
    k_move_pass(SysPtrs p1, const SysPtrs *reps, const int *gstart, const int *rep_ids, int n_reps, int pass,
                int *pool0, int *pool1, long long pool_cells) {
  static_assert(G == 1 || G == 2 || G == 4 || G == 8, "group size");
  // Launched as a programmatic dependent of the previous pass (launch_gc),
  // the blocks become resident while that pass drains and wait here until it
  // has completed and its writes are visible; nothing is read before.  The
  // next pass may then be scheduled (once every block of this one runs).
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PassSm m = pass_smem_ptrs<G, CAP>(smem_raw);
  const int tid = (int)threadIdx.x;
  const int lane = tid % G;
  const int gl = tid / G;  // group within the block
  const int col0 = tid - lane;
  const int group = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);
  const int gbase = (tid & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  PassTally t;

  if (!BATCH) {
    const SysPtrs &p = p1;
    const unsigned long long sweep = p.st->params.sweep;
    const int layout = (int)(sweep & 1ull);
    PassEnv e = pass_env(p, 0u, layout);
    e.seq = sweep * 8ull + (unsigned long long)pass;
    const int colour = p.st->params.perm[pass];
    // The first pass of a sweep clears the other layout for the next build.
    if (pass == 0) {
      int *other = cnt_of(p, layout ^ 1);
      for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x)
        other[c] = 0;
    }
    const int groups = (int)((gridDim.x * blockDim.x) / G);
    const int hx = e.nc[0] >> 1, hy = e.nc[1] >> 1, hz = e.nc[2] >> 1;
    const int n_active = hx * hy * hz;
    const int cx = colour & 1, cy = (colour >> 1) & 1, cz = (colour >> 2) & 1;
    for (int ac = group; ac < n_active; ac += groups) {
      if (G > 1) __syncwarp(gmask);  // the previous cell's records are no longer read
      const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
      move_cell<G, CAP, TRACE, false>(e, m, tid, lane, gl, col0, gmask, 2 * ax + cx, 2 * ay + cy, 2 * az + cz, t);
    }
    add_tally(t, p.st);
    return;
  }

  if (pass == 0 && pool_cells > 0) {
    const int layout0 = (int)(reps[0].st->params.sweep & 1ull);
    int *other = layout0 ? pool0 : pool1;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < pool_cells;
         c += (long long)gridDim.x * blockDim.x)
      other[c] = 0;
  }
  int r = -1;
  if (group < __ldg(gstart + n_reps)) {
    r = find_rep(gstart, n_reps, group);
    const SysPtrs p = reps[r];
    const unsigned long long sweep = p.st->params.sweep;
    PassEnv e = pass_env(p, (uint32_t)__ldg(rep_ids + r), (int)(sweep & 1ull));
    e.seq = sweep * 8ull + (unsigned long long)pass;
    const int colour = p.st->params.perm[pass];
    const int hx = e.nc[0] >> 1, hy = e.nc[1] >> 1;
    const int ac = group - __ldg(gstart + r);
    const int ax = ac % hx, ayz = ac / hx, ay = ayz % hy, az = ayz / hy;
    move_cell<G, CAP, TRACE, false>(e, m, tid, lane, gl, col0, gmask, 2 * ax + (colour & 1),
                                    2 * ay + ((colour >> 1) & 1), 2 * az + ((colour >> 2) & 1), t);
  }
  // the lanes of one replica sum their counters together
  const cg::thread_block_tile<32> tile = cg::tiled_partition<32>(cg::this_thread_block());
  const auto part = cg::labeled_partition(tile, r);
  const unsigned a = cg::reduce(part, t.acc, cg::plus<unsigned>());
  const unsigned o = cg::reduce(part, t.rej_o, cg::plus<unsigned>());
  const unsigned bnd = cg::reduce(part, t.rej_b, cg::plus<unsigned>());
  const unsigned rc = cg::reduce(part, t.rechecks, cg::plus<unsigned>());
  if (r >= 0 && part.thread_rank() == 0) {
    DevState *ws = reps[r].st;
    if (a) atomicAdd(&ws->acc, (unsigned long long)a);
    if (o) atomicAdd(&ws->rej_overlap, (unsigned long long)o);
    if (bnd) atomicAdd(&ws->rej_boundary, (unsigned long long)bnd);
    if (rc) atomicAdd(&ws->rechecks, (unsigned long long)rc);
  }
}

// All eight passes of a sweep in one cooperative launch, without barriers
// between passes.  The grid is cut into 2x2x2 regions, one cell of each
// colour; a group owns regions and goes through its regions pass by pass.
// Before pass k of a cell it waits until the seven regions around the
// cell's own have published pass k - 1 (prog[r] = 8 sweep + passes done),
// so each cell sees its 26 neighbours exactly as after the pass barrier: the
// chain is the one of k_move_pass.  The wait is per warp (all its groups'
// neighbourhoods), so the groups of a warp stay converged.  Waits only point
// from pass k to pass k - 1 and every block is resident (cooperative launch),
// so the schedule cannot deadlock; each wait is bounded and reports
// ST_FLOW_TIMEOUT.
__device__ __forceinline__ void warp_wait(const uint32_t *prog, const int *reg, bool valid, uint32_t target,
                                          int *status) {
  uint64_t t0 = 0;
  for (;;) {
    bool ready = true;
    if (valid) {
#pragma unroll
      for (int k = 0; k < 7; k++) ready &= (int)(ld_acquire(prog + reg[k]) - target) >= 0;
    }
    if (__all_sync(0xffffffffu, ready)) break;
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    if (t0 == 0) t0 = t;
    if (__any_sync(0xffffffffu, t - t0 > 1000000000ull)) {
      if ((threadIdx.x & 31) == 0) atomicOr(status, ST_FLOW_TIMEOUT);
      break;
    }
    __nanosleep(64);
  }
  __threadfence();
}

template <int G, int CAP, bool TRACE>
__global__ void __launch_bounds__(128, PassSmem<G, CAP>::min_blocks) k_move_flow(SysPtrs p, uint32_t *prog) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const PassSm m = pass_smem_ptrs<G, CAP>(smem_raw);
  const unsigned long long sweep = p.st->params.sweep;
  const int layout = (int)(sweep & 1ull);
  PassEnv e = pass_env(p, 0u, layout);

  {
    int *other = cnt_of(p, layout ^ 1);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.ncell_alloc; c += gridDim.x * blockDim.x) other[c] = 0;
  }

  const int tid = (int)threadIdx.x;
  const int lane = tid % G;
  const int gl = tid / G;
  const int col0 = tid - lane;
  const int group = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G);
  const int groups = (int)((gridDim.x * blockDim.x) / G);
  const int gbase = (tid & 31) & ~(G - 1);
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << gbase);
  const int hx = e.nc[0] >> 1, hy = e.nc[1] >> 1, hz = e.nc[2] >> 1;
  const int n_active = hx * hy * hz;
  const int iters = (n_active + groups - 1) / groups;  // the same for every thread
  const uint32_t base = (uint32_t)(sweep * 8ull);
  const int hold = p.st->flow_hold;

  PassTally t;
  for (int pass = 0; pass < 8; pass++) {
    const int colour = p.st->params.perm[pass];
    const int cx = colour & 1, cy = (colour >> 1) & 1, cz = (colour >> 2) & 1;
    e.seq = sweep * 8ull + (unsigned long long)pass;
    for (int it = 0; it < iters; it++) {
      const int ac = group + it * groups;
      const bool valid = ac < n_active;
      const int acv = valid ? ac : 0;
      const int ax = acv % hx, ayz = acv / hx, ay = ayz % hy, az = ayz / hy;
      if (pass > 0) {
        // the regions holding the cell's neighbours: its own and, per axis,
        // the one on the side the cell sits
        int reg[7];
        const int bx = cx ? (ax + 1 == hx ? 0 : ax + 1) : (ax == 0 ? hx - 1 : ax - 1);
        const int by = cy ? (ay + 1 == hy ? 0 : ay + 1) : (ay == 0 ? hy - 1 : ay - 1);
        const int bz = cz ? (az + 1 == hz ? 0 : az + 1) : (az == 0 ? hz - 1 : az - 1);
#pragma unroll
        for (int q = 1; q < 8; q++) {
          const int rx = (q & 1) ? bx : ax, ry = (q & 2) ? by : ay, rz = (q & 4) ? bz : az;
          reg[q - 1] = rx + hx * (ry + hy * rz);
        }
        warp_wait(prog, reg, valid, base + (uint32_t)pass, &p.st->status);
      }
      if (valid)
        move_cell<G, CAP, TRACE, true>(e, m, tid, lane, gl, col0, gmask, 2 * ax + cx, 2 * ay + cy, 2 * az + cz, t);
      __syncwarp();
      if (valid && lane == 0 && ac != hold) {
        __threadfence();
        st_release(prog + ac, base + (uint32_t)pass + 1u);
      }
    }
  }
  add_tally(t, p.st);
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

template <int G, int CAP, bool TRACE>
static void allow_flow_smem() {
  if (pass_smem<G, CAP>() > (size_t)smem_optin_limit()) return;
  cudaFuncSetAttribute(k_move_flow<G, CAP, TRACE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)pass_smem<G, CAP>());
}

template <int G, int CAP>
static void allow_all() {
  allow_smem<G, CAP, false, false>();
  allow_smem<G, CAP, true, false>();
  allow_smem<G, CAP, false, true>();
  allow_flow_smem<G, CAP, false>();
  allow_flow_smem<G, CAP, true>();
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

template <int G>
static size_t smem_for_g(int cap) {
  return cap <= 8 ? PassSmem<G, 8>::bytes : (cap <= 16 ? PassSmem<G, 16>::bytes : PassSmem<G, 32>::bytes);
}

static size_t smem_for(int group, int cap) {
  switch (group) {
    case 1: return smem_for_g<1>(cap);
    case 2: return smem_for_g<2>(cap);
    case 4: return smem_for_g<4>(cap);
    default: return smem_for_g<8>(cap);
  }
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

// A pass is a programmatic dependent launch: it may be scheduled before the
// kernel ahead of it in the stream has finished, and waits for it inside
// (griddepcontrol.wait), which hides the launch latency between passes.
template <int G, int CAP>
static void launch_gc(const SysPtrs &p, int pass, bool trace, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = pass_smem<G, CAP>();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const SysPtrs *no_reps = nullptr;
  const int *no_ints = nullptr;
  int *no_pool = nullptr;
  if (trace)
    cudaLaunchKernelEx(&cfg, k_move_pass<G, CAP, true, false>, p, no_reps, no_ints, no_ints, 0, pass, no_pool, no_pool,
                       0ll);
  else
    cudaLaunchKernelEx(&cfg, k_move_pass<G, CAP, false, false>, p, no_reps, no_ints, no_ints, 0, pass, no_pool,
                       no_pool, 0ll);
}

template <int G, int CAP>
static void launch_batch_gc(const SysPtrs *reps, const int *gstart, const int *ids, int n_reps, int tot_groups,
                            int pass, int *pool0, int *pool1, long long pool_cells, cudaStream_t s) {
  const long long threads = (long long)tot_groups * G;
  const int grid = (int)((threads + 127) / 128);
  k_move_pass<G, CAP, false, true><<<grid > 0 ? grid : 1, 128, pass_smem<G, CAP>(), s>>>(
      SysPtrs{}, reps, gstart, ids, n_reps, pass, pool0, pool1, pool_cells);
}

void launch_move_pass_batch(const SysPtrs *reps, const int *gstart, const int *ids, int n_reps, int tot_groups,
                            int cap, int pass, int group, int *cnt_pool0, int *cnt_pool1, long long pool_cells,
                            cudaStream_t s) {
#define HSMC_BATCH_CAP(G)                                                                                  \
  switch (cap) {                                                                                           \
    case 8: launch_batch_gc<G, 8>(reps, gstart, ids, n_reps, tot_groups, pass, cnt_pool0, cnt_pool1, pool_cells, s); break; \
    case 16: launch_batch_gc<G, 16>(reps, gstart, ids, n_reps, tot_groups, pass, cnt_pool0, cnt_pool1, pool_cells, s); break; \
    default: launch_batch_gc<G, 32>(reps, gstart, ids, n_reps, tot_groups, pass, cnt_pool0, cnt_pool1, pool_cells, s); break; \
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

// Dataflow sweep: the grid is every block the device can hold at once (the
// cooperative launch checks it), so every group's waits can be met.
template <int G, int CAP>
static int flow_blocks_for(int num_sms) {
  if (pass_smem<G, CAP>() > (size_t)smem_optin_limit()) return 0;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_move_flow<G, CAP, false>, 128, pass_smem<G, CAP>());
  int per_sm_t = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_t, k_move_flow<G, CAP, true>, 128, pass_smem<G, CAP>());
  if (per_sm_t < per_sm) per_sm = per_sm_t;
  return per_sm * num_sms;
}

template <int G>
static int flow_blocks_g(int cap, int num_sms) {
  switch (cap) {
    case 8: return flow_blocks_for<G, 8>(num_sms);
    case 16: return flow_blocks_for<G, 16>(num_sms);
    default: return flow_blocks_for<G, 32>(num_sms);
  }
}

int move_flow_grid(int group, int cap, int ncell_alloc, int num_sms) {
  int cap_blocks = 0;
  switch (group) {
    case 1: cap_blocks = flow_blocks_g<1>(cap, num_sms); break;
    case 2: cap_blocks = flow_blocks_g<2>(cap, num_sms); break;
    case 4: cap_blocks = flow_blocks_g<4>(cap, num_sms); break;
    default: cap_blocks = flow_blocks_g<8>(cap, num_sms); break;
  }
  const long long threads = (long long)(ncell_alloc / 8) * group;  // one group per region at most
  const int need = (int)((threads + 127) / 128);
  return need < cap_blocks ? (need > 0 ? need : 1) : cap_blocks;
}

template <int G, int CAP, bool TRACE>
static cudaError_t launch_flow_gct(const SysPtrs &p, uint32_t *prog, int grid, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(128);
  cfg.dynamicSmemBytes = pass_smem<G, CAP>();
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_move_flow<G, CAP, TRACE>, p, prog);
}

template <int G>
static cudaError_t launch_flow_g(const SysPtrs &p, uint32_t *prog, bool trace, int grid, cudaStream_t s) {
  switch (p.cap) {
    case 8: return trace ? launch_flow_gct<G, 8, true>(p, prog, grid, s) : launch_flow_gct<G, 8, false>(p, prog, grid, s);
    case 16:
      return trace ? launch_flow_gct<G, 16, true>(p, prog, grid, s) : launch_flow_gct<G, 16, false>(p, prog, grid, s);
    default:
      return trace ? launch_flow_gct<G, 32, true>(p, prog, grid, s) : launch_flow_gct<G, 32, false>(p, prog, grid, s);
  }
}

cudaError_t launch_move_flow(const SysPtrs &p, uint32_t *prog, int group, bool trace, int grid, cudaStream_t s) {
  switch (group) {
    case 1: return launch_flow_g<1>(p, prog, trace, grid, s);
    case 2: return launch_flow_g<2>(p, prog, trace, grid, s);
    case 4: return launch_flow_g<4>(p, prog, trace, grid, s);
    default: return launch_flow_g<8>(p, prog, trace, grid, s);
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
