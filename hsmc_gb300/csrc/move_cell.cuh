// The trial moves of one active cell by a group of G lanes (part_move /
// check_overlap, src/moves.c:27-80 and 157-212), shared by the colour-pass
// kernels (move_pass.cu) and the persistent batched sweep (batch_persist.cu).
//
// A group of G lanes owns one active cell at a time; the 26 neighbour cells
// are split across the lanes and the lanes agree on each decision with one
// ballot.  Per cell:
//   counts      of the cell and of the lane's neighbour cells, issued together;
//   own data    the cell's slots, its particles' ranks by id and their FP64
//               coordinates (nothing before the cell's own pass writes them);
//   neighbours  every slot of the neighbour cells copied with cp.async into
//               the group's pool in shared memory (one column per lane, so
//               each lane screens an equal share); the lanes then add the
//               periodic image to the pool entries they copied.
// Then n trials (n = particles in the cell), each on the particle of rank
// floor(u n) by id: FP64 proposal (its axes shared out over the group's
// lanes), confinement to the cell, single-precision screen four candidates at
// a time, FP64 re-evaluation of any pair within the guard band of contact.
// Nothing per cell lives in local memory.
#pragma once

#include "screen.cuh"

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
  bool signal;  // a colour pass: let the next pass launch once the neighbours are copied
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
// schedule, the persistent batched sweep) must bypass the non-coherent L1:
// FLOW selects the L2-only forms (counts, slots and FP64 coordinates).
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
// wait_prev: the group has not yet waited for the previous pass (this pass
// is its programmatic dependent).  The cell's own data (counts, its slots,
// its particles' FP64 coordinates) is loaded first, and only then does the
// group wait, before the neighbours' slots, which the previous pass writes;
// wait_prev is cleared once it has.  An empty cell returns without waiting.
template <int G, int CAP, bool TRACE, bool FLOW>
__device__ __forceinline__ void move_cell(const PassEnv &e, const PassSm &m, int tid, int lane, int gl, int col0,
                                          unsigned gmask, int ix, int iy, int iz, PassTally &t, bool &wait_prev) {
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
  const int n = FLOW ? __ldcg(e.cnt + c) : e.cnt[c];
#pragma unroll
  for (int q = 0; q < NB; q++) {
    const int mm = (lane + q * G < 26) ? (FLOW ? __ldcg(e.cnt + nb_c[q]) : e.cnt[nb_c[q]]) : 0;
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

  // (2) the cell's own slots, its particles' ranks by id (the chain must
  // not depend on the order the build's atomics filled the slots) and their
  // FP64 coordinates.  No pass writes a cell but the cell's own colour's,
  // and the counts change only at the build, so none of this depends on the
  // previous pass.
  for (int j = lane; j < n; j += G) copy16<FLOW>(&m.own_t[j * GPB + gl], e.slot + (size_t)c * CAP + j);
  cp_async_wait_all();
  if (G > 1) __syncwarp(gmask);
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
  // the first trial's draws
  U32x4 r_next = draw4(e.seed, e.rep << 8, (uint32_t)c, e.seq, TAG_MOVE);
  if (wait_prev) {
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    wait_prev = false;
  }

  // (3) the neighbours' slots, copied asynchronously into the pool.  Entry
  // e sits in column e % G of its group; in phase ph each lane copies only
  // the entries of column (lane + ph) % G, so the lanes of a group never
  // write the same bank column in one instruction.
  if (!direct) {
    if (G == 2 || G == 4) {
#pragma unroll 1
      for (int ph = 0; ph < G; ph++) {  // not unrolled: the smaller code measured 0.5 % faster
        const int col = (lane + ph) & (G - 1);
        int k0 = first;
#pragma unroll
        for (int q = 0; q < NB; q++) {
          const Slot *src = e.slot + (size_t)nb_c[q] * CAP;
          for (int k = (col - k0) & (G - 1); k < nb_n[q]; k += G)
            copy16<FLOW>(&m.pool[((k0 + k) / G) * 128 + col0 + col], src + k);
          k0 += nb_n[q];
        }
      }
    } else {
      int k0 = first;
#pragma unroll
      for (int q = 0; q < NB; q++) {
        const Slot *src = e.slot + (size_t)nb_c[q] * CAP;
        for (int k = 0; k < nb_n[q]; k++, k0++) copy16<FLOW>(&m.pool[(k0 / G) * 128 + col0 + k0 % G], src + k);
      }
    }
  }
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
  // The next pass's blocks may take free block slots from here on: started
  // earlier, their loads would compete with this pass's neighbour copies.
  if (e.signal) asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");

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
          const int mm = FLOW ? __ldcg(e.cnt + nbc) : e.cnt[nbc];
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
  e.signal = false;
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

}  // namespace hsmc
