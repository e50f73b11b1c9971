/*
 * hsmc_gpu.h -- C ABI of the GB300 (sm_103a) hard-sphere Monte Carlo engine.
 *
 * This is the boundary a host program in C calls in place of the HSMC
 * reference's local-move hot path.  Plain pointers and sizes only; every call
 * is synchronous on the context's own CUDA stream and returns 0 (HSMC_OK) or
 * one of the error codes below.  hsmc_gpu_strerror() gives the reference's
 * message for an error, so a host shim can print it and exit as the
 * reference does.
 *
 * Ownership: the device owns positions, the cell layout and the random stream
 * between calls.  Host buffers are always caller-owned; the host-side
 * configuration keeps the reference's double[N][4] layout (id, x, y, z)
 * (src/sim_info.h:20), so write_config / write_restart work unchanged on a
 * downloaded copy.
 *
 * Threading: one host thread per context.  A process may hold several
 * contexts (independent systems).
 *
 * Reference interfaces each entry point replaces are cited beside it
 * (paths relative to the reference project).
 */
#ifndef HSMC_GPU_H
#define HSMC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- errors */
enum hsmc_status {
  HSMC_OK = 0,
  HSMC_ERR_INVALID_ARG = 1,   /* bad size, pointer or parameter */
  HSMC_ERR_CUDA = 2,          /* a CUDA runtime call failed */
  HSMC_ERR_NO_DEVICE = 3,     /* no usable sm_103 device */
  HSMC_ERR_CELL_OVERFLOW = 4, /* more particles in one cell than it holds (src/cell_list.c:228-231) */
  HSMC_ERR_CELL_TOO_SMALL = 5,/* box too small for the cell grid (src/cell_list.c:126-129) */
  HSMC_ERR_BAD_BIN = 6,       /* a pair fell outside its histogram (r < 1: overlapping input) */
  HSMC_ERR_TIMEOUT = 7,       /* a bounded device wait gave up */
  HSMC_ERR_OUT_OF_BOX = 8,    /* a coordinate outside [0, L] on upload */
  HSMC_ERR_OVERLAP = 9,       /* the configuration contains an overlapping pair */
  HSMC_ERR_CAVITY_RANGE = 10  /* the cavities' distance left [cavity_mindr, cavity_maxdr]
                                 before a cavity move (src/moves.c:288-297) */
};

typedef struct hsmc_ctx hsmc_ctx;

/* Parameters of one system.  The box is the reference's rectangular periodic
 * box (src/sim_info.c:32-71); n_particles and the lattice counts follow its
 * input keywords (src/read_input.c:138-192). */
typedef struct {
  int n_particles;      /* N */
  int lattice_type;     /* 1 = simple cubic, 2 = FCC (keyword "type") */
  int cells[3];         /* lattice cell counts (keywords cells_x/y/z) */
  double rho;           /* number density (keyword "rho") */
  double box[3];        /* box sides lx, ly, lz */
  double dr_max;        /* maximum particle displacement (keyword "dr_max") */
  double dv_max;        /* maximum ln V change for NpT (keyword "npt", 2nd value) */
  double pressure;      /* beta*P for NpT, 0 for NVT (keyword "npt", 1st value) */
  uint64_t seed;        /* random stream key (keyword "seed") */
  int cell_capacity;    /* particles per device cell; 0 chooses from the cell size */
  int lanes_per_cell;   /* GPU lanes sharing one active cell in a move pass: 1, 2, 4 or 8;
                           0 picks the default; 1 is refused for 32-slot cells (its
                           shared memory does not fit a block) */
  double min_cell_edge; /* NVT only: smallest edge of the device cells (0 = 1 plus the rounding
                           margin).  Larger cells hold more spheres each; for a sparse fluid an
                           edge near rho^(-1/3) spreads the per-cell cost over about one sphere.
                           Part of the chain's definition, like the seed. */
  double cavity_pcav;   /* cavity sampling (keyword "cavity", src/cavity_nvt.c): > 0 turns it on;
                           NVT only.  Particles 0 and 1 are the cavities; see hsmc_gpu_sweeps */
  double cavity_maxdr;  /* largest and smallest allowed distance between the cavities */
  double cavity_mindr;
  int reserved[4];
} hsmc_params;

/* Replaces the set-up in hs_nvt / hs_npt (src/nvt.c:30-62, src/npt.c:25-70):
 * allocates device state for one system.  Positions start undefined; call
 * hsmc_gpu_upload_config next. */
int hsmc_gpu_create(const hsmc_params *params, hsmc_ctx **out);

/* Frees everything the context holds (src/nvt.c:97-100). */
void hsmc_gpu_destroy(hsmc_ctx *ctx);

/* Copies a host configuration double[n][4] = (id, x, y, z) to the device and
 * builds the cell layout (src/cell_list.c:142-175).  conf[i][0] must equal i
 * (else HSMC_ERR_INVALID_ARG) and coordinates must lie in [0, L] (else
 * HSMC_ERR_OUT_OF_BOX); both are checked on the device after the copy, and
 * a configuration that fails leaves the context without one: the calls that
 * need a configuration return HSMC_ERR_INVALID_ARG until an upload
 * succeeds. */
int hsmc_gpu_upload_config(hsmc_ctx *ctx, const double (*conf)[4], int n);

/* Copies the device configuration back into double[n][4]
 * (the array part_config_get returns, src/sim_info.c:187-190). */
int hsmc_gpu_download_config(hsmc_ctx *ctx, double (*conf)[4], int n);

/* Sets the maximum displacement and volume step (G_IN.dr_max / G_IN.dv_max,
 * written by the optimiser, src/optimizer.c:23-166). */
int hsmc_gpu_set_step(hsmc_ctx *ctx, double dr_max, double dv_max);

/* The reference's optimiser in one call (opt_nvt src/optimizer.c:23-64,
 * opt_npt :83-148 for an NpT context, opt_cavity_nvt :172-212 for a cavity
 * run): opt_samples + 2 samples of opt_sweeps / opt_samples sweeps each, the
 * step after the first sample doubled or halved toward part_target (and
 * vol_target for the volume step), then secant steps with the reference's
 * clamps.  The samples run back to back on the device, which sets the step
 * for each next sample itself; the host waits once.  The steps and
 * acceptances are the reference's double arithmetic on the same counters,
 * so the result is the host-side loop's bit for bit.
 * out (may be NULL): {dr_max, last particle acceptance, dv_max, last volume
 * acceptance (0 for NVT)}; the context keeps the new steps. */
int hsmc_gpu_optimize(hsmc_ctx *ctx, int opt_sweeps, int opt_samples, double part_target, double vol_target,
                      double out[4]);

/* Counter order used by the sweep calls: the six move counters of
 * get_moves_counters (src/moves.c:231-241), 64-bit, for this call only. */
enum {
  HSMC_CNT_MOVES = 0,
  HSMC_CNT_ACCEPTED = 1,
  HSMC_CNT_REJECTED = 2,
  HSMC_CNT_VOL_MOVES = 3,
  HSMC_CNT_VOL_ACCEPTED = 4,
  HSMC_CNT_VOL_REJECTED = 5
};

/* NVT: n_sweeps sweeps of N trial moves each (sweep_nvt, src/nvt.c:201-209,
 * part_move src/moves.c:27-80).  counters may be NULL. */
int hsmc_gpu_sweeps(hsmc_ctx *ctx, int n_sweeps, uint64_t counters[6]);

/* NpT: n_sweeps sweeps, each N trial particle moves and one trial volume
 * move on average (sweep_npt, src/npt.c:177-196; vol_move src/moves.c:83-153). */
int hsmc_gpu_npt_sweeps(hsmc_ctx *ctx, int n_sweeps, uint64_t counters[6]);

/* Current box: out[0..2] = lx, ly, lz, out[3] = volume, out[4] = density
 * (sim_box_info_get, src/sim_info.c:179-181; G_IN.rho after volume moves). */
int hsmc_gpu_get_box(hsmc_ctx *ctx, double out[5]);

/* g(r) pair counts before normalisation (rdf_hist_compute,
 * src/compute_rdf.c:110-128): counts[b] = number of ordered pairs (i, j != i)
 * with r < rmax and (int)((r - 1)/dr) == b, which equals the reference's
 * histogram value (2 per unordered pair).  rmax must already be the adjusted
 * cutoff dr*nbins + 1 (src/compute_rdf.c:104) and at most half the box. */
int hsmc_gpu_rdf(hsmc_ctx *ctx, double dr, double rmax, int nbins, uint64_t *counts);

/* hsmc_gpu_rdf without any allocation, for callers that cannot let the
 * library allocate device memory: a program that gives all device memory to
 * its own memory manager up front or runs under a fixed memory budget on a
 * shared GPU, or a sampling loop that cannot absorb a first-call cudaMalloc.
 * No counterpart in the reference.  The counts use a fixed device array of
 * HSMC_RDF_NOALLOC_MAX_BINS 64-bit bins compiled into the library (resident
 * on every GPU that loads it until the process exits); more bins are refused
 * with HSMC_ERR_INVALID_ARG.  The first call on a device looks up that
 * array's device address, so make the first call before any stream capture.
 * All calls share the array and clear it before counting: calls that run at
 * the same time on one GPU race on it.  Results equal hsmc_gpu_rdf's. */
#define HSMC_RDF_NOALLOC_MAX_BINS 16384
int hsmc_gpu_rdf_noalloc(hsmc_ctx *ctx, double dr, double rmax, int nbins, uint64_t *counts);

/* Host helper, no device work: the squared distances at which the bin of
 * rdf_hist_compute / pressv_compute_hist (src/compute_rdf.c:110-128,
 * src/compute_press.c:123-165), (int)((sqrt(r2) - 1) / dr), steps up.
 * thr[0] = 1; thr[k] (k = 1..nbins) is the smallest double r2 whose bin is
 * at least k; thr[nbins + 1] the smallest whose root reaches rmax.  For
 * every double r2 in [1, thr[nbins]) the bin is the largest k with
 * thr[k] <= r2.  The pair counts use them to bin pairs exactly without the
 * square root and division; thr holds nbins + 2 doubles. */
int hsmc_pair_thresholds(double dr, double rmax, int nbins, double *thr);

/* Virial-route contact histogram, the same counting on [1, rmax)
 * (pressv_compute_hist, src/compute_press.c:123-165). */
int hsmc_gpu_pressv(hsmc_ctx *ctx, double dr, double rmax, int nbins, uint64_t *counts);

/* Thermodynamic route: for each scale factor sf[k] < 1, nonoverlap[k] = 1 when
 * no pair overlaps with all distances scaled by sf[k], else 0
 * (presst_compute_hist, src/compute_press.c:243-273; sf = (1 - xi)^(1/3)
 * computed by the caller as the reference does). */
int hsmc_gpu_presst(hsmc_ctx *ctx, const double *sf, int n_sf, uint64_t *nonoverlap);

/* Full scaled overlap scan of a trial volume move (src/moves.c:104-112):
 * *overlap = 1 when any pair is closer than 1 after scaling by sf. */
int hsmc_gpu_scan_overlap(hsmc_ctx *ctx, double sf, int *overlap);

/* Widom test-particle insertions at uniform points (widom_insertion,
 * src/compute_widom_chem_pot.c:44-71): *accepted = insertions without overlap.
 * The host forms mu = -ln(accepted/n) as the reference does. */
int hsmc_gpu_widom(hsmc_ctx *ctx, int64_t n_insertions, uint64_t *accepted);

/* Mean Steinhardt q_l over all particles (global_ql_compute,
 * src/compute_order_parameter.c:82-94); rc is the bond cutoff after the
 * reference's clipping to its cell size (src/compute_order_parameter.c:31-40).
 * per_particle may be NULL or an array of N doubles. */
int hsmc_gpu_ql(hsmc_ctx *ctx, int l, double rc, double *ql_mean, double *per_particle);

/* Random stream position for restart files, replacing the GSL state block of
 * write_restart / read_restart (src/io_config.c:61-62, 115-116):
 * state[0] = seed, state[1] = sweeps done, state[2] = Widom calls done,
 * state[3] = cluster moves done. */
int hsmc_gpu_rng_state(hsmc_ctx *ctx, uint64_t out[4]);
int hsmc_gpu_rng_set_state(hsmc_ctx *ctx, const uint64_t state[4]);

/* Reference message for a status code (the printf text the reference emits
 * before exit(EXIT_FAILURE)); never NULL. */
const char *hsmc_gpu_strerror(int status);

/* --------------------------------------------------------- cavity sampling
 * Torrie-Patey cavity simulations (cavity_hs_nvt, cavity_part_move,
 * cavity_check_move; src/cavity_nvt.c, src/moves.c:254-440).  A context
 * created with cavity_pcav > 0 treats particles 0 and 1 as the cavities:
 * they overlap nothing but each other's umbrella potential
 * psi(r) = ln y_GH(r) (Grundke-Henderson over Verlet-Weis and Percus-Yevick,
 * src/analytic.c:34-230, at packing fraction pi rho / 6), and every other
 * particle treats them as hard spheres.  Each sweep of hsmc_gpu_sweeps is the
 * checkerboard sweep of the other particles (a trial that picks a cavity
 * leaves it in place) followed by round(N * cavity_pcav) cavity trials in
 * sequence, each accepted with probability min(1, exp(-(psi(r') - psi(r))))
 * when the new distance lies in [cavity_mindr, cavity_maxdr] and the moved
 * cavity overlaps no other particle.  The uniforms are the context's
 * counter-based stream; psi uses the device's FP64 exp, cos, sin and log.
 * The move counters include the cavity trials.
 *
 * hsmc_gpu_cavity_psi evaluates psi at n distances on the device (the
 * values the moves use).  hsmc_gpu_cavity_trace starts (capacity > 0) or
 * stops (0) recording every cavity trial of the following sweeps, 8 words
 * each: sweep (low 32 bits), trial, cavity, the three step draws, the
 * acceptance draw, decision (0 accepted, 1 out of the distance range, 2
 * rejected by the Metropolis test, 3 overlap); hsmc_gpu_cavity_trace_read
 * copies the records out and clears them. */
int hsmc_gpu_cavity_psi(hsmc_ctx *ctx, const double *x, int n, double *out);
int hsmc_gpu_cavity_trace(hsmc_ctx *ctx, int64_t capacity);
int hsmc_gpu_cavity_trace_read(hsmc_ctx *ctx, uint32_t *rec, int64_t capacity, int64_t *n_rec);

/* ---------------------------------------------------------- cluster moves
 * Geometric cluster moves (cluster_move / cluster_move_part / pocket_add,
 * src/cluster_nvt.c:232-410; Dress & Krauth, J. Phys. A 28, L597, 1995):
 * a pivot point and a coordinate axis are drawn, and the seed particle is
 * rotated by pi about the line through the pivot along that axis with the
 * reference's rotate() arithmetic (src/cluster_nvt.c:342-365, cos and sin of
 * M_PI as the host's libm gives them), then wrapped once into the box
 * (apply_pbc).  Every particle that overlaps a moved particle joins the
 * cluster and is moved the same way, until none overlaps.  The move is
 * always accepted.  The reference grows the cluster from a randomly ordered
 * pocket; the device grows it breadth-first over the whole GPU.  Both give
 * the same set of moved particles and bit-identical positions: the rotation
 * is an isometry, so a moved particle never overlaps another moved one.
 *
 * hsmc_gpu_cluster_moves makes n_moves moves with pivot, axis and seed drawn
 * from the context's random stream.  sizes (n_moves entries, or NULL)
 * receives each cluster's size (the reference's cluster_size); drawn
 * (5 x n_moves doubles, or NULL) receives pivot x, y, z, axis (0 = x, 1 = y,
 * 2 = z) and seed particle of each move.
 * hsmc_gpu_cluster_move_at makes one move with the given pivot, axis and
 * seed particle and does not advance the stream.
 * Both are NVT only (HSMC_ERR_INVALID_ARG on an NpT context).  A wait of the
 * device-wide breadth-first search that runs out (1 s) is HSMC_ERR_TIMEOUT. */
int hsmc_gpu_cluster_moves(hsmc_ctx *ctx, int n_moves, int64_t *sizes, double *drawn);
int hsmc_gpu_cluster_move_at(hsmc_ctx *ctx, const double pivot[3], int axis, int seed_particle, int64_t *size);

/* ------------------------------------------------------ batched replicas
 * Many independent NVT systems (different N, box and density) advanced
 * together: every kernel of a sweep covers all replicas in one launch, and
 * sweeps run as one CUDA graph.  Replica k's chain is the chain a context
 * with the same parameters would run, except that k enters its random
 * counters; replica 0 of a batch reproduces a single context exactly.
 * Each system is the reference's single-system NVT run (hs_nvt,
 * src/nvt.c:30-199); the batch has no reference counterpart. */
typedef struct hsmc_batch hsmc_batch;

int hsmc_batch_create(const hsmc_params *params, int n_systems, hsmc_batch **out);
void hsmc_batch_destroy(hsmc_batch *b);
int hsmc_batch_upload_config(hsmc_batch *b, int k, const double (*conf)[4], int n);
int hsmc_batch_download_config(hsmc_batch *b, int k, double (*conf)[4], int n);
int hsmc_batch_set_steps(hsmc_batch *b, const double *dr_max);
/* counters: n_systems x 6 in the order of hsmc_gpu_sweeps (may be NULL) */
int hsmc_batch_sweeps(hsmc_batch *b, int n_sweeps, uint64_t *counters);
/* virial contact counts of every replica: counts[k * nbins + bin], with
 * rmax = dr * nbins + 1 as hsmc_gpu_pressv takes it */
int hsmc_batch_pressv(hsmc_batch *b, double dr, double rmax, int nbins, uint64_t *counts);
/* device time of the last hsmc_batch_sweeps call, in milliseconds */
int hsmc_batch_last_timing(hsmc_batch *b, double *total_ms);

/* Schedule of hsmc_batch_sweeps.  0 (the default): every sweep is a cell
 * build and eight colour passes, each one flat launch over the replicas of
 * one cell capacity, in CUDA graphs of 8 sweeps.  1: persistent, every sweep
 * of a call in one launch (per cell capacity) of thread-block clusters of
 * cluster_blocks blocks (1, 2, 4, 8), captured in a CUDA graph: the replicas
 * are packed into bundles of about tile x (lane groups of a cluster) active
 * cells (tile 1..64; at most 32 replicas per bundle), one cluster per bundle,
 * which runs all the call's sweeps of its replicas with the cluster's
 * hardware barrier between the build and the passes; bundles never wait on
 * one another.  2: persistent, every sweep of a call in one cooperative
 * launch (per cell capacity) of every block the device holds: each sweep's
 * cell build and eight colour passes over all the replicas' cells, separated
 * by grid-wide barriers whose waits give up after 1 s (HSMC_ERR_TIMEOUT);
 * cluster_blocks and tile are kept but not used.  3: the flat launches of 0,
 * with each pass's cells (over every replica of a cell capacity) listed
 * fullest first after the build, so a warp's cells hold the same number of
 * spheres and empty cells take no lanes (two more launches per capacity and
 * sweep).  The chain is the same in all four (sweep_nvt, src/nvt.c:201-209,
 * per replica).
 * HSMC_ERR_INVALID_ARG for a cluster shape the device cannot hold, or a
 * device without cooperative launches.  get_schedule: out = {schedule,
 * cluster_blocks, tile}. */
int hsmc_batch_set_schedule(hsmc_batch *b, int schedule, int cluster_blocks, int tile);
int hsmc_batch_get_schedule(hsmc_batch *b, int out[3]);

/* Times schedules 0, 3 and 2, and schedule 1 with every cluster size (1, 2,
 * 4, 8) and tile (1, 2, 4), over sweeps_per_variant sweeps each, after an
 * untimed call of 8 sweeps, and keeps the fastest (out as get_schedule).
 * These are ordinary sweeps of every replica's chain. */
int hsmc_batch_autotune(hsmc_batch *b, int sweeps_per_variant, int out[3]);

/* ----------------------------------------------------- replay and checks
 * Entry points that evaluate the reference's decisions on given inputs
 * without advancing the chain.  They exist so a caller (or a test) can compare
 * decisions with the reference's own code on the same proposals. */

/* Overlap decision of check_overlap (src/moves.c:157-212) for particle ids[k]
 * placed at pos[3k..3k+2], each against the current configuration (no
 * update between entries).  overlap[k] = 1 when rejected. */
int hsmc_gpu_overlap_replay(hsmc_ctx *ctx, const int *ids, const double *pos, int n, uint8_t *overlap);

/* Widom decisions (widom_check_overlap, src/compute_widom_chem_pot.c:82-120)
 * for insertion points pos[3k..3k+2]. */
int hsmc_gpu_widom_replay(hsmc_ctx *ctx, const double *pos, int n, uint8_t *overlap);

/* Sweeps that also record every trial move:
 * rec[k] = {pass, cell, trial, id, draw_x, draw_y, draw_z, decision,
 *           shift_x, shift_y, shift_z (float bits), flags}
 * (12 x uint32 per move; decision 0 accepted, 1 overlap, 2 left its cell).
 * capacity is in records; *n_rec receives the count (HSMC_ERR_INVALID_ARG if
 * it would exceed capacity). */
int hsmc_gpu_sweeps_traced(hsmc_ctx *ctx, int n_sweeps, uint32_t *rec, int64_t capacity, int64_t *n_rec,
                           uint64_t counters[6]);

/* Geometry of the device cell grid used by the sweeps: nc[3], len32[3] and
 * inv_w32[3] (float), capacity; for checking traced moves. */
int hsmc_gpu_grid_info(hsmc_ctx *ctx, int nc[3], float len32[3], float inv_w32[3], int *capacity);

/* Times every schedule (below) with every lanes-per-cell mapping (1, 2, 4,
 * 8) over sweeps_per_variant sweeps each (rounded up to a multiple of 8),
 * twice over in two rounds, each timed run after an untimed graph's worth of
 * sweeps, and keeps the variant with the fastest run; *lanes_out receives
 * its mapping.  The chain depends on neither (same random counters, exact
 * decisions), so these are ordinary sweeps of the run: 2 x (8 + S) sweeps
 * per variant. */
int hsmc_gpu_autotune(hsmc_ctx *ctx, int sweeps_per_variant, int *lanes_out);

/* Schedule of the eight colour passes of a sweep: 0 = one launch per pass
 * with a kernel boundary between passes; 1 = dataflow, all eight passes in
 * one cooperative launch where a cell waits only for the 26 cells around it
 * to finish the previous pass; 2 = one block, every sweep of a call in one
 * launch with the system in shared memory (systems of up to a few thousand
 * spheres, NVT or NpT with its volume move per sweep; the default up to 128
 * active cells per pass, about 1000 spheres, where it is faster); 3 = as 0,
 * but each pass hands out its colour's non-empty cells fullest first, so a
 * warp's cells hold the same number of spheres (two more launches per
 * sweep; the default where a pass has more active cells than one wave of
 * 2-lane groups, else 0).  All give the same
 * chain; hsmc_gpu_autotune picks the fastest.  lanes_per_cell 0 keeps the
 * current mapping (schedule 2 has none; it also runs a cavity run's cavity
 * stage).  Traced and profiled sweeps, and cavity runs recording their
 * trials, use schedule 0 or 1. */
int hsmc_gpu_set_schedule(hsmc_ctx *ctx, int schedule, int lanes_per_cell);
int hsmc_gpu_get_schedule(hsmc_ctx *ctx, int *schedule, int *lanes_per_cell);

/* Diagnostic of the dataflow schedule's bounded waits: region (a 2x2x2
 * block of cells, index x + hx (y + hy z) over the half-grid) stops
 * publishing its progress, so every wait on it runs out after 1 s and the
 * sweep returns HSMC_ERR_TIMEOUT; -1 restores normal operation (and the
 * progress words).  The context stays usable throughout. */
int hsmc_gpu_hold_region(hsmc_ctx *ctx, int region);

/* Timing of the last sweep or observable call (g(r), pressure scans, Widom,
 * q_l), from CUDA events on the context's stream around its kernels: total
 * device time, and (for sweeps with profiling on) the summed time and count
 * of the move-pass kernel launches.  With profiling on, sweeps are launched
 * one kernel at a time instead of as a CUDA graph, with one event pair around
 * the eight move passes of each sweep (the passes keep their programmatic
 * dependent launches); move_launches counts the passes so bracketed. */
int hsmc_gpu_set_profiling(hsmc_ctx *ctx, int on);
int hsmc_gpu_last_timing(hsmc_ctx *ctx, double *total_ms, double *move_kernel_ms, int *move_launches);

/* ------------------------------------------------------------------------
 * Learned Widom proposal: an importance-sampled form of compute_mu
 * (src/compute_widom_chem_pot.c:32-182); no counterpart in the reference.
 *
 * Insertion points are drawn from q(x) = alpha / V + (1 - alpha) q_L(x):
 * q_L picks a sub-cell (edge >= subcell_edge, at most 1/sqrt(3) so that a
 * sub-cell holds at most one sphere) with probability proportional to
 * pi_c = sqrt(sigmoid(z_c)) and a point uniformly inside it, where z_c is
 * the output of an MLP 27 -> 64 -> 64 -> 1 (BF16 tensor-core products, FP32
 * accumulation) on the 27 occupancy bits of the sub-cell's 3x3x3
 * neighbourhood.  Each point carries w = 1 / (V q(x)); the mean of
 * w * [no overlap] estimates the insertion probability without bias, and
 * beta mu_ex = -ln of it.  The overlap test is the reference's FP64 test.
 * The network is trained on insertion outcomes the sampler itself collects
 * (pattern bits | success << 31), with weighted binary cross-entropy and
 * Adam.  All calls are synchronous on the context's stream. */
typedef struct hsmc_lwidom hsmc_lwidom;

#define HSMC_LWIDOM_NPARAMS 6273 /* W1[64][32] (column 27 = bias), W2[64][64], b2[64], w3[64], b3 */

typedef struct {
  double sum_w;       /* sum of w over successful insertions */
  double sum_w2;      /* sum of w^2 over successful insertions */
  uint64_t n;         /* insertions */
  uint64_t n_ok;      /* successful insertions */
  uint64_t n_learned; /* insertions drawn from the learned component */
} hsmc_lwidom_stats;

/* train_capacity: outcomes the training buffer holds (0 = none).  The
 * proposal runs on ctx's stream and reads its cells: destroy it before ctx. */
int hsmc_lwidom_create(hsmc_ctx *ctx, double subcell_edge, uint64_t seed, int64_t train_capacity,
                       hsmc_lwidom **out);
void hsmc_lwidom_destroy(hsmc_lwidom *lw);
int hsmc_lwidom_set_params(hsmc_lwidom *lw, const float *params); /* also resets Adam */
int hsmc_lwidom_get_params(hsmc_lwidom *lw, float *params);
int hsmc_lwidom_subgrid(hsmc_lwidom *lw, int ns[3]);
/* Occupancy, patterns, logits and the proposal CDF for the context's
 * current configuration; required before insertions on it. */
int hsmc_lwidom_refresh(hsmc_lwidom *lw);
int hsmc_lwidom_patterns(hsmc_lwidom *lw, uint32_t *out, int64_t n_subcells);
int hsmc_lwidom_proposal(hsmc_lwidom *lw, double *pi, double *cdf, int64_t n_subcells);
/* Network output for given patterns (replaces the refreshed logits). */
int hsmc_lwidom_logits(hsmc_lwidom *lw, const uint32_t *patterns, int64_t n, float *logits);
/* Gradient of the mean weighted loss over samples (pattern | label << 31),
 * weight w_pos for label 1 and w_neg for label 0; *loss = the mean loss. */
int hsmc_lwidom_grad(hsmc_lwidom *lw, const uint32_t *samples, int64_t n, float w_pos, float w_neg, float *grad,
                     double *loss);
/* One Adam step (b1 0.9, b2 0.999, eps 1e-8) with the given gradient. */
int hsmc_lwidom_adam_step(hsmc_lwidom *lw, const float *grad, float lr);
/* n insertions with mixture weight alpha in (0, 1].  keep_failures >= 0
 * appends outcomes to the training buffer while it has room: every success,
 * and each failure with probability keep_failures (an independent draw), so
 * failures are trained with weight 1 / keep_failures; < 0 collects nothing.
 * Collected outcomes land in the buffer in atomic-claim order. */
int hsmc_lwidom_insert(hsmc_lwidom *lw, int64_t n, double alpha, double keep_failures, hsmc_lwidom_stats *st);
/* The same, returning every point, its learned sub-cell (-1 for a uniform
 * draw), branch, weight and outcome. */
int hsmc_lwidom_insert_traced(hsmc_lwidom *lw, int64_t n, double alpha, double *points, int32_t *subcell,
                              uint8_t *uniform, double *weight, uint8_t *ok, hsmc_lwidom_stats *st);
/* Plain uniform Widom (the reference's estimator) through the same overlap
 * test and timing; *accepted = successful insertions. */
int hsmc_lwidom_uniform(hsmc_lwidom *lw, int64_t n, uint64_t *accepted);
/* Minibatch Adam over the collected outcomes, loss weight w_pos for
 * successes and w_neg for failures; *last_loss = mean weighted loss of the
 * last minibatch. */
int hsmc_lwidom_train(hsmc_lwidom *lw, int epochs, int64_t batch, float lr, float w_pos, float w_neg,
                      double *last_loss);
int hsmc_lwidom_samples(hsmc_lwidom *lw, int64_t *n, int64_t *n_pos);
int hsmc_lwidom_clear_samples(hsmc_lwidom *lw);
/* Device time of the last refresh, insert, uniform or train call (ms). */
int hsmc_lwidom_last_timing(hsmc_lwidom *lw, double *ms);

#ifdef __cplusplus
}
#endif

#endif
