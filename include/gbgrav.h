/*
 * gbgrav.h — C ABI of the GB300 self-gravity engine (sm_103a CUDA).
 *
 * Drop-in boundary for the acceleration call of the reference's
 * Engine(gravity_mode="direct"|"bh") (Khaserdene/real-astronomy-simulation,
 * core/engine.py:101-106).  Each entry point names the reference function it
 * replaces.
 *
 * Conventions
 *  - Particle arrays are device pointers to float4 records, passed as float*
 *    (4 floats per particle, 16-byte aligned):
 *      xm  = {x, y, z, m}    positions and masses
 *      vel = {vx, vy, vz, 0} velocities
 *      acc = {ax, ay, az, 0} accelerations
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Every call
 *    is stream-ordered and asynchronous unless stated otherwise.
 *  - Every function returns a status code (GB_OK = 0); the message for the
 *    last failure on the calling thread is gb_last_error_string().
 *  - Handles are not thread-safe: one thread (or external locking) per
 *    handle.  The caller owns particle buffers; handles own their scratch.
 */
#ifndef GBGRAV_H
#define GBGRAV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GB_OK 0
#define GB_EINVAL 1     /* bad argument (size, pointer, alignment) */
#define GB_ENOMEM 2     /* device allocation failed */
#define GB_ESTACK 3     /* traversal stack rule dropped work (see gb_diag_t) */
#define GB_ETIMEOUT 4   /* a bounded device wait expired */
#define GB_ECUDA 5      /* CUDA runtime error */
#define GB_ENOTREADY 6  /* call order violated (e.g. accel before build) */

/* Flags */
#define GB_ACCUMULATE 0x1  /* acc += result instead of acc = result */
#define GB_PLAIN_FP32 0x2  /* plain FP32 accumulation (no Kahan compensation) */
#define GB_COUNT_WORK 0x4  /* tree traversal also counts its work (gb_diag_t) */
#define GB_USE_GRAPH 0x8   /* KDK calls: replay captured steps as a CUDA graph */
#define GB_CHECK 0x10      /* tree calls: wait for the call and fail on counted failures */

/* Device diagnostic counters, read back by gb_*_diag (synchronising). */
typedef struct gb_diag {
    uint64_t stack_drops;     /* pushes skipped by the max_stack rule */
    uint64_t stack_overflow;  /* warp stack capacity reached */
    uint64_t nonfinite;       /* non-finite positions met while keying */
    uint64_t bad_tree;        /* inconsistent index met (never for a valid tree) */
    /* Traversal work, counted only by calls with GB_COUNT_WORK: */
    uint64_t warp_node_reads;   /* 48-byte two-children node records read (per warp) */
    uint64_t warp_root_reads;   /* 32-byte root records read (per warp) */
    uint64_t lane_interactions; /* monopole terms summed (per particle) */
    uint64_t lane_tests;        /* acceptance tests evaluated (per particle) */
    uint64_t wait_timeouts;     /* bounded device waits that gave up (the sort's
                                   look-back; never expected): GB_ETIMEOUT */
} gb_diag_t;

const char *gb_last_error_string(void);
int gb_version(void);

/* ------------------------------------------------------------ direct N^2 */
typedef struct gb_direct gb_direct_t;

/* Allocates scratch for systems of up to n_max particles on the current
 * device.  Replaces the Taichi field allocation in Engine.load_state
 * (core/engine.py:66-69). */
int gb_direct_create(gb_direct_t **out, int64_t n_max);
int gb_direct_destroy(gb_direct_t *h);

/* Tile shape: k targets per lane (2 or 4), warps per CTA (4 or 8), CTAs per
 * SM (0 = occupancy maximum).  Chosen by the autotuner. */
int gb_direct_set_tiles(gb_direct_t *h, int k, int warps, int ctas_per_sm);

/* Inner-loop form: 0 = scalar FP32 (default), 1 = packed .f32x2 FP32, one
 * pass per target; 2 = symmetric packed .f32x2, each unordered pair once,
 * applied to both particles.  The symmetric pass keeps 8 KB slots per
 * 512 x 512 tile pair (N^2/32 bytes in all at large N); above the band
 * budget (gb_direct_set_sym_band, 1 GiB by default) it runs in bands of tile
 * rows, two kernels per band, plus 32 bytes per particle of running sums.
 * Same results up to FP32 rounding order.  gb_direct_phi (and gb_energy)
 * follow the variant too: form 2 sums each pair's potential once for both
 * particles. */
int gb_direct_set_variant(gb_direct_t *h, int packed);

/* Tile-pair slot bytes per band of the symmetric pass (at least 40 KB:
 * one tile pair with four source slices).  Measurement and testing knob; the
 * default, 1 GiB, keeps a band's slots in a small share of HBM. */
int gb_direct_set_sym_band(gb_direct_t *h, int64_t bytes);

/* acc_i = G sum_j m_j (x_j - x_i) / (|x_j - x_i|^2 + eps2)^{3/2}, all j
 * (i == j adds zero).  Replaces compute_acc_direct
 * (core/solvers/gravity.py:13-26); the GB_ACCUMULATE flag gives the
 * `acc +=` form of grav_self_direct (core/living_galaxy_engine.py:102-114). */
int gb_direct_acc(gb_direct_t *h, const float *xm, float *acc, int64_t n,
                  float G, float eps2, int flags, void *stream);

/* nsteps kick-drift-kick leapfrog steps with direct forces, in place.
 * acc must hold the accelerations of the current positions on entry.
 * Replaces Engine.step (core/engine.py:108-116) with kick/drift
 * (core/integrators/leapfrog.py:11-22) fused into the force pass.  With
 * GB_USE_GRAPH a run of 8 steps and a single step are captured as CUDA graphs
 * (again whenever the pointers, n, a parameter, the tile shape or the pass
 * change) and replayed, whole runs first: identical results, less launch
 * overhead at small n. */
int gb_direct_kdk(gb_direct_t *h, float *xm, float *vel, float *acc, int64_t n,
                  float G, float eps2, float dt, int64_t nsteps, int flags,
                  void *stream);

/* Standalone leapfrog halves on n float4 records, for callers that step
 * outside the fused KDK path: vel += acc * dt_half (kick, core/integrators/
 * leapfrog.py:11-15) and xm.xyz += vel * dt (drift, :18-22; the mass column
 * is untouched).  Same FMA forms as the fused step, so kick -> drift ->
 * gb_direct_acc -> kick equals gb_direct_kdk bit for bit. */
int gb_kick(float *vel, const float *acc, int64_t n, float dt_half, void *stream);
int gb_drift(float *xm, const float *vel, int64_t n, float dt, void *stream);

/* phi_i = sum_{j != i} m_j / sqrt(|x_j - x_i|^2 + eps2) (FP32, Kahan): the
 * inner sum of potential_energy (core/solvers/gravity.py:47-55). */
int gb_direct_phi(gb_direct_t *h, const float *xm, float *phi, int64_t n,
                  float eps2, int flags, void *stream);

/* FP64 energies into out3 (3 doubles): kinetic, potential, total.
 * KE = 1/2 sum m v^2 (core/solvers/gravity.py:29-36); PE = -1/2 G sum m_i
 * phi_i (core/solvers/gravity.py:39-57) with phi from gb_direct_phi; the
 * reductions run in FP64 in a fixed order, in one launch.  n = 0 writes
 * zeros (xm and vel may then be NULL).  out3 in device memory: the call is
 * asynchronous.  out3 in host memory (pinned, or pageable): the call copies
 * the three sums there and waits for the stream before it returns (the
 * energy calls' synchronous form, for a caller that reads them at once;
 * not for use while the stream is being captured). */
int gb_energy(gb_direct_t *h, const float *xm, const float *vel, int64_t n,
              float G, float eps2, double *out3, void *stream);

/* The potential as an epilogue of the force pass: gb_direct_acc /
 * gb_direct_kdk that also write phi (n floats, device) with the same sums
 * gb_direct_phi returns, phi_i = sum_{j != i} m_j / sqrt(|x_j - x_i|^2 +
 * eps2) (no G), of the positions the pass evaluated (for the KDK call: the
 * positions after its last step; earlier steps run without it).  The pair
 * loop forms m_j / |d| for the force anyway: the potential costs one FMA per
 * pair side in the symmetric form and one add per pair in the per-target
 * forms, plus the particle's own term, which the per-target fix-up
 * subtracts.  Replaces the separate O(N^2) potential_energy pass
 * (core/solvers/gravity.py:39-57) that the reference's callers run at every
 * print (core/simulation.py:112-114, core/sim_controller.py:287-293). */
int gb_direct_acc_phi(gb_direct_t *h, const float *xm, float *acc, float *phi,
                      int64_t n, float G, float eps2, int flags, void *stream);
int gb_direct_kdk_phi(gb_direct_t *h, float *xm, float *vel, float *acc,
                      float *phi, int64_t n, float G, float eps2, float dt,
                      int64_t nsteps, int flags, void *stream);

/* Accelerations of the targets t0 .. t0 + nt - 1 from all n sources of xm
 * into acc[0 .. nt) (nt float4 records), and, when phi is not NULL, their
 * potential sums into phi[0 .. nt): one slice of the target loop
 * `for i in range(n)` of compute_acc_direct (core/solvers/gravity.py:18-26),
 * the unit a rank computes when the targets are split across GPUs (each
 * rank holds all n positions, gathered once per step).  Runs the handle's
 * per-target pass (the scalar pass when the variant is 2); flags
 * GB_ACCUMULATE and GB_PLAIN_FP32.  Each target sums the same terms as in
 * gb_direct_acc; the stream-K split of the work differs, so results agree
 * with a whole-system call to FP32 rounding of the Kahan-compensated sums. */
int gb_direct_acc_range(gb_direct_t *h, const float *xm, int64_t n,
                        int64_t t0, int64_t nt, float *acc, float *phi,
                        float G, float eps2, int flags, void *stream);

/* gb_energy with phi given (from an epilogue above, or gb_bh_accel_phi):
 * only the O(n) FP64 reductions run, KE = 1/2 sum m v^2, PE = -1/2 G sum m
 * phi (core/solvers/gravity.py:29-57).  out3 as in gb_energy (device:
 * asynchronous; host: copied there, the call waits). */
int gb_energy_phi(gb_direct_t *h, const float *xm, const float *vel,
                  const float *phi, int64_t n, float G, double *out3,
                  void *stream);

/* FP64 oracle on the device for sampled targets: acc_out (nt x 3 doubles)
 * = compute_acc_direct (core/solvers/gravity.py:13-26) in float64 for the
 * particles listed in targets. */
int gb_direct_acc_fp64(const float *xm, int64_t n, const int64_t *targets,
                       int64_t nt, double G, double eps2, double *acc_out,
                       void *stream);

int gb_direct_diag(gb_direct_t *h, gb_diag_t *out, int reset);

/* Kernels launched through this handle so far (host-side count; measurement
 * support, no reference counterpart). */
uint64_t gb_direct_launch_count(gb_direct_t *h);

/* ----------------------------------------------------- LBVH Barnes-Hut */
typedef struct gb_bh gb_bh_t;

/* Allocates tree scratch for up to n_max particles (1 .. 2^30 - 1) with
 * key_bits bits per axis (21: the reference's 63-bit keys,
 * core/solvers/barnes_hut.py:38; 10: 30-bit keys).  Replaces
 * BarnesHut.__init__ (core/solvers/barnes_hut.py:223-240). */
int gb_bh_create(gb_bh_t **out, int64_t n_max, int key_bits);
int gb_bh_destroy(gb_bh_t *h);

/* Device build: bounding box, Morton keys (bit-identical to morton_codes,
 * core/solvers/barnes_hut.py:27-46), stable radix sort (the permutation of
 * np.argsort(kind="stable"), :247), Karras tree (_build_radix, :84-121),
 * node summaries (_leaf_init/_accumulate/_finalize, :124-177). */
int gb_bh_build(gb_bh_t *h, const float *xm, int64_t n, void *stream);

/* Accelerations from the last build: _traverse (core/solvers/barnes_hut.py:
 * 180-217) with the same acceptance test and max_stack rule; pushes that the
 * rule skips are counted in gb_diag_t.stack_drops (the reference drops them
 * silently, :212).  With GB_CHECK in flags (or gb_bh_set_check on) the call
 * waits for its stream and fails when failure counters grew since the last
 * checked call on the handle (or the last diag reset): GB_ESTACK for pushes
 * dropped by the max_stack rule or lost to the traversal stack's capacity,
 * GB_EINVAL for non-finite positions or an inconsistent tree, GB_ETIMEOUT
 * when a bounded wait of the build's radix sort expired (never expected).
 * The results are written either way. */
int gb_bh_accel(gb_bh_t *h, float *acc, float theta, float eps2, float G,
                int max_stack, int flags, void *stream);

/* gb_bh_accel that also writes the tree potential of every particle into
 * phi (n floats, device, no G): the monopole terms m / sqrt(|d|^2 + eps2) of
 * the nodes the traversal accepts for the force, the particle's own leaf
 * excluded.  It approximates the potential_energy sum
 * (core/solvers/gravity.py:47-55) within the tree's own error (the
 * reference has no tree potential and always runs the O(N^2) sum). */
int gb_bh_accel_phi(gb_bh_t *h, float *acc, float *phi, float theta,
                    float eps2, float G, int max_stack, int flags,
                    void *stream);

/* gb_bh_accel (or, with phi not NULL, gb_bh_accel_phi) for the targets at
 * key-order positions s0 .. s0 + ns - 1 of the last build only: each one's
 * acceleration is written to acc at its particle index (the other records
 * of acc are left as they are), with exactly the node visits of the full
 * call, so the values are bit-identical to it.  In the group walk (traversal
 * shape 3) the range covers the groups whose first leaf lies in it.  A rank
 * that owns one slice of the key order after a replicated build runs this on
 * a zeroed acc; an all-reduce (sum) of the ranks' acc then gives every
 * particle its acceleration exactly, each sum having one non-zero term.
 * Flags: GB_ACCUMULATE, GB_CHECK.  One slice of the traversal loop over all
 * particles of core/solvers/barnes_hut.py:180-217, 257-259. */
int gb_bh_accel_range(gb_bh_t *h, float *acc, float *phi, int64_t s0,
                      int64_t ns, float theta, float eps2, float G,
                      int max_stack, int flags, void *stream);

/* build + accel: BarnesHut.compute (core/solvers/barnes_hut.py:242-259). */
int gb_bh_compute(gb_bh_t *h, const float *xm, float *acc, int64_t n,
                  float theta, float eps2, float G, int max_stack, int flags,
                  void *stream);

/* nsteps KDK steps with tree forces, in place (Engine.step with the BH
 * solver, core/engine.py:101-116); kick and drift are fused into the first
 * tree stage and the closing kick into the traversal.  With
 * gb_bh_set_check on, the call waits for the steps and reports failures
 * counted during them as gb_bh_accel does with GB_CHECK. */
int gb_bh_kdk(gb_bh_t *h, float *xm, float *vel, float *acc, int64_t n,
              float theta, float eps2, float G, float dt, int64_t nsteps,
              int max_stack, void *stream);

/* gb_bh_kdk whose last step also writes the tree potential of the final
 * positions into phi (as gb_bh_accel_phi); the earlier steps run without
 * it.  The step with the potential is captured as a graph of its own. */
int gb_bh_kdk_phi(gb_bh_t *h, float *xm, float *vel, float *acc, float *phi,
                  int64_t n, float theta, float eps2, float G, float dt,
                  int64_t nsteps, int max_stack, void *stream);

/* FP64 energies from a tree potential (gb_energy_phi on the tree handle's
 * scratch): KE, PE = -1/2 G sum m phi, total into out3 (3 doubles; device:
 * asynchronous; host: copied there, the call waits). */
int gb_bh_energy(gb_bh_t *h, const float *xm, const float *vel,
                 const float *phi, int64_t n, float G, double *out3,
                 void *stream);

/* gb_bh_kdk replays one captured step as a CUDA graph (on = 1, default)
 * instead of launching its kernels one by one (on = 0).  The graph is
 * captured on the first call and again whenever the pointers, n or a
 * parameter change; results are identical (measured 13% faster per step
 * at N = 3,000, 6% at 100,000, 1% at 1,000,000).  While stage timing
 * (gb_bh_timing) is on, the kernels are launched directly. */
int gb_bh_set_graph(gb_bh_t *h, int on);

/* Failure checks on every tree call of the handle (on = 1), as the GB_CHECK
 * flag gives one call: gb_bh_accel, gb_bh_accel_ext, gb_bh_compute and
 * gb_bh_kdk wait for their stream and return GB_ESTACK / GB_EINVAL /
 * GB_ETIMEOUT when failure counters grew.  Off (0) by default: the calls stay asynchronous.
 * No reference counterpart (its stack rule drops work silently,
 * core/solvers/barnes_hut.py:212). */
int gb_bh_set_check(gb_bh_t *h, int on);

/* Copies one array of the last build, in the reference's layout, to device
 * memory dst: 0 codes (uint64[n], key order), 1 order (int32[n]), 2 left,
 * 3 right (int32[n-1]), 4 parent (int32[2n-1]), 5 mass (double[2n-1]),
 * 6 com, 7 min, 8 max (double[2n-1][3]); nodes are leaves 0..n-1 then
 * internal nodes n..2n-2 as in core/solvers/barnes_hut.py:229-240. */
int gb_bh_export(gb_bh_t *h, int what, void *dst, void *stream);

int gb_bh_diag(gb_bh_t *h, gb_diag_t *out, int reset);

/* Traversal shape.  1 and 2: warp-coherent, the warp's 32 (or 64, two per
 * lane) key-consecutive targets walk the tree together, one node record per
 * warp step.  0: per lane, each lane walks its own target with its own
 * stack (max_stack <= 127 and n <= 2^25 + 1; otherwise mode 1 runs).  -1
 * (default): 0 below n = 131,072, 1 from there.  All modes give
 * bit-identical results: each target meets its nodes in the same order.
 * Mode 1 is fastest on the 1M disk (per-lane record loads diverge); mode 0
 * on small systems, where a warp-coherent launch has too few warps to hide
 * each step's latency.
 * 3 (opt-in): group walk.  The targets are cut into groups, the largest
 * subtrees with at most 32 leaves; a group accepts a node when
 * size^2 < theta^2 (dmin^2 + eps^2), dmin the distance from the node's
 * centre of mass to the group's bounding box, so every target of the group
 * passes the reference's own test (core/solvers/barnes_hut.py:204-210) on
 * every accepted node: each target sums a refinement of its per-particle
 * node set, with force errors no larger on the 1M disk (median 0.84 %
 * against 0.94 %) in about a third of the traversal time.  The node sets
 * differ from the per-particle walk's, so results are not bit-identical to
 * modes -1..2; the max_stack rule does not apply (a full group stack takes
 * the child as a monopole and counts it in stack_overflow).  Keys, order and
 * topology are the same in every mode. */
int gb_bh_set_traversal(gb_bh_t *h, int targets_per_lane);

/* Stage timing for measurement: with timing enabled, every build/step records
 * CUDA events on its stream at the boundaries of the GB_BH_STAGES stages
 * (0 bbox+keys, 1 sort, 2 gather+Karras, 3 summaries, 4 traversal).
 * gb_bh_stage_times synchronises, returns the summed milliseconds per stage
 * over the (at most GB_BH_TIMING_STEPS) steps since the last call, and the
 * step count.  gb_bh_launch_count returns the kernels this handle launched.
 * No reference counterpart (measurement support). */
#define GB_BH_STAGES 5
#define GB_BH_TIMING_STEPS 64
int gb_bh_timing(gb_bh_t *h, int enable);
int gb_bh_stage_times(gb_bh_t *h, float *ms, int *steps);
uint64_t gb_bh_launch_count(gb_bh_t *h);

/* ------------------------------------------------ batched direct N^2 */
/* Many independent systems of uneven size, concatenated in one set of
 * float4 arrays (system s occupies particles off[s] .. off[s+1]-1 with off
 * the prefix sum of sizes).  Each system is integrated exactly like
 * Engine(gravity_mode="direct").step (core/engine.py:108-116) on its own;
 * the reference has no batched form. */
typedef struct gb_batch gb_batch_t;

/* sizes: host array of nsys system sizes (each >= 1). */
int gb_batch_create(gb_batch_t **out, const int64_t *sizes, int nsys);
int gb_batch_destroy(gb_batch_t *h);
/* Same meaning as gb_direct_set_tiles; chosen by the autotuner. */
int gb_batch_set_tiles(gb_batch_t *h, int k, int warps, int ctas_per_sm);
/* Force-pass form: 0 = one pass per target (default); 1 = symmetric packed
 * .f32x2 (each unordered pair of a system once, both particles updated; the
 * same tile-pair pass as gb_direct_set_variant 2, over all systems in one
 * launch from an atomic unit counter).  Selecting 1 allocates its scratch
 * (about 16 KB per 512 x 512 tile pair of every system) and fails with
 * GB_EINVAL above 3 GiB of it.  Same results up to FP32 rounding order. */
int gb_batch_set_variant(gb_batch_t *h, int variant);
int64_t gb_batch_total(gb_batch_t *h);

/* Direct accelerations of every system (compute_acc_direct per system,
 * core/solvers/gravity.py:13-26), one persistent launch for all systems. */
int gb_batch_acc(gb_batch_t *h, const float *xm, float *acc, float G,
                 float eps2, int flags, void *stream);

/* nsteps KDK steps of every system, in place; acc must hold the current
 * accelerations.  One persistent force launch + one fix-up launch per step;
 * with GB_USE_GRAPH the nsteps loop is captured once as a CUDA graph (kept
 * until the pointers, parameters or tiles change) and replayed. */
int gb_batch_kdk(gb_batch_t *h, float *xm, float *vel, float *acc, float G,
                 float eps2, float dt, int64_t nsteps, int flags,
                 void *stream);

/* The same steps as a loop over systems of the single-system call
 * gb_direct_kdk (two launches per system and step): the plain alternative
 * the batched launch is measured against. */
int gb_batch_kdk_loop(gb_batch_t *h, float *xm, float *vel, float *acc,
                      float G, float eps2, float dt, int64_t nsteps,
                      int flags, void *stream);
uint64_t gb_batch_launch_count(gb_batch_t *h);

/* --------------------------------------------------------------- adjoint */
/* One reverse-mode step of the direct-sum KDK leapfrog (gb_direct_kdk),
 * hand-written; the reference has no gradients.  xm holds the positions and
 * masses at which the step evaluated its forces (the step's output
 * positions).  On entry lx, lv, la are the adjoints of the step's outputs
 * x', v', a'; on return they are the adjoints of its inputs x, v, a, and
 * lm (n floats) has the step's mass gradient added:
 *   w = la + (dt/2) lv;  (gx, gm) = VJP of the force at xm with w;
 *   lx += gx;  lv += dt lx;  la = (dt/2) lv;  lm += gm.
 * prime = 1 instead applies the priming force evaluation a0 = F(x0)
 * (Engine.load_state, core/engine.py:81): w = la, lx += gx, lm += gm. */
int gb_adjoint_step(gb_direct_t *h, const float *xm, float *lx, float *lv,
                    float *la, float *lm, int64_t n, float G, float eps2,
                    float dt, int prime, void *stream);

/* Pair evaluation of the adjoint:
 *   2 (default) every unordered pair once, applied to both particles, in
 *     packed FP32x2 arithmetic with CTAs taking tile-pair units from a
 *     counter (8 KB slots per 512 x 512 tile pair, allocated on first use;
 *     above the handle's band budget, gb_direct_set_sym_band, it runs in
 *     bands of tile rows with 16 bytes per particle of running sums);
 *   1 every unordered pair once, scalar FP32, static runs per CTA (scratch
 *     about n^2 / 32 bytes; above 3 GiB of it the call runs form 0);
 *   0 each ordered pair, one pass per target (no extra scratch).
 * All are deterministic; they differ by FP32 summation order. */
int gb_adjoint_set_variant(gb_direct_t *h, int variant);

/* ------------------------------------------------- allocation-free call */
/* No counterpart in the reference.  gb_direct_acc without a handle and
 * without any device allocation, for callers that cannot call cudaMalloc:
 * an application whose memory pool owns the whole GPU, a plug-in running in
 * another framework's memory arena, or a loop that must never block
 * (cudaMalloc/cudaFree can synchronise the device).  Same arguments and
 * result as gb_direct_acc; only the flags GB_ACCUMULATE and GB_PLAIN_FP32
 * apply, and any other flag bit is rejected with GB_EINVAL.  The caller
 * still passes xm and acc.  Scratch is a 4 MiB file-scope device array that
 * every GPU loading the library keeps until the process exits; it holds the
 * partial sums of systems of at most GB_NOALLOC_MAX_N particles, and larger
 * n is rejected with GB_EINVAL.  The first call on each device looks up the
 * array's device address (with that device current) and caches it; make
 * that first call before any stream capture.  A cudaDeviceReset of a device
 * invalidates the cached address: do not call this entry point on a device
 * after resetting it.  All calls on a device share the array: calls whose
 * kernels overlap on the GPU (other streams or host threads) race and must
 * be ordered by the caller. */
#define GB_NOALLOC_MAX_N 65536
#define GB_NOALLOC_MAX_DEVICES 64
int gb_direct_acc_noalloc(const float *xm, float *acc, int64_t n, float G,
                          float eps2, int flags, void *stream);

/* ---------------------------------------------- analytic galaxy potential */
/* The fixed analytic potential that the living-galaxy and gas-disk engines
 * add after self-gravity (grav_analytic, core/living_galaxy_engine.py:
 * 124-151; add_analytic, core/gas_disk_engine.py:54-81): a Miyamoto-Nagai
 * disk (mass M_d, scale lengths a, b), a Hernquist (is_hernquist = 1) or
 * Plummer (0) halo (M_h, a_h) and, when smbh_mass > 0, a point mass at the
 * origin softened as in the reference.  Same fields as the engines' `pot`
 * dict; masses in the units of G.  Evaluated in FP32 with G folded into the
 * masses. */
typedef struct gb_potential {
    double M_d, a, b, M_h, a_h, smbh_mass;
    int32_t is_hernquist;
    int32_t reserved; /* must be 0 */
} gb_potential_t;

/* acc += the potential's acceleration at every particle (acc = it without
 * GB_ACCUMULATE): grav_analytic / add_analytic, for callers whose
 * self-gravity comes from elsewhere. */
int gb_analytic_acc(const float *xm, float *acc, int64_t n, float G,
                    const gb_potential_t *pot, int flags, void *stream);

/* gb_direct_acc with the potential added in the same pass that writes the
 * results (the fix-up).  With GB_ACCUMULATE this is add_grav_ext
 * (core/gas_disk_engine.py:20-51), and grav_self_direct followed by
 * grav_analytic (core/living_galaxy_engine.py:1016-1027).  pot = NULL gives
 * gb_direct_acc. */
int gb_direct_acc_ext(gb_direct_t *h, const float *xm, float *acc, int64_t n,
                      float G, float eps2, const gb_potential_t *pot,
                      int flags, void *stream);

/* gb_bh_accel with the potential added in the traversal's epilogue: the
 * tree branch of the engines' force pass, BarnesHut.compute + add_field /
 * add_acc + add_analytic / grav_analytic (core/gas_disk_engine.py:216-225,
 * core/living_galaxy_engine.py:1013-1027), with GB_ACCUMULATE.  pot = NULL
 * gives gb_bh_accel. */
int gb_bh_accel_ext(gb_bh_t *h, float *acc, float theta, float eps2, float G,
                    int max_stack, const gb_potential_t *pot, int flags,
                    void *stream);

/* ------------------------------------------------- SPH neighbour grid */
/* Uniform grid over the gas particles for the SPH neighbour walk, rebuilt on
 * the device: NeighborGrid (core/solvers/neighbor_grid.py:35-136), whose
 * rebuild the reference runs in host numpy.  Outputs are bit-identical to
 * the reference's for the same float32 inputs: gsort (gas indices in stable
 * cell order, zero-padded to n) and cell_start (max_cells + 1 entries, cell
 * c's first slot in gsort for c <= n_cells, zero above), with
 * max_cells = max(64, 4 n) and the cell size max(2 h_max, min_radius) grown
 * by 1.3 until the grid fits. */
typedef struct gb_grid gb_grid_t;

typedef struct gb_grid_info {
    int64_t ngas, n_cells;
    int32_t nx, ny, nz;
    int32_t status;       /* 0 ok, 1 non-finite input, 2 no fitting grid */
    double lo[3], cell, inv_cell;
} gb_grid_info_t;

/* NeighborGrid.__init__(n, min_radius) (:38-48): scratch for n particles. */
int gb_grid_create(gb_grid_t **out, int64_t n, double min_radius);
int gb_grid_destroy(gb_grid_t *h);
/* max(64, 4 n): cell_start needs max_cells + 1 entries. */
int64_t gb_grid_max_cells(gb_grid_t *h);

/* rebuild (is_star != NULL; gas = is_star == 0) or rebuild_all (is_star =
 * NULL; every particle is gas) (:49-136).  xm: n float4 {x, y, z, m};
 * hsml: n smoothing lengths; is_star: n int32; gsort: int32[max(n, 1)];
 * cell_start: int32[max_cells + 1] (device, caller-owned, like the
 * reference's fields).  Asynchronous on `stream`; a rebuild without gas
 * leaves gsort, cell_start and the geometry unchanged, as the reference
 * does.  When info is not NULL the call waits for the stream and fills it
 * (the reference's return value ngas and its nx, ny, nz, lo, inv_cell), and
 * a non-finite gas position or smoothing length returns GB_EINVAL (an
 * expired bounded wait of the radix sort, never expected, GB_ETIMEOUT). */
int gb_grid_rebuild(gb_grid_t *h, const float *xm, const float *hsml,
                    const int32_t *is_star, int32_t *gsort, int32_t *cell_start,
                    gb_grid_info_t *info, void *stream);

/* Kernels launched through this handle (measurement support). */
uint64_t gb_grid_launch_count(gb_grid_t *h);

/* Test support for the bounded waits: runs the radix sort's look-back of
 * one 256-thread CTA for tile 1 of a fresh two-tile status array.
 * publish_first = 1: tile 0's prefix is published first (digit d's count =
 * d), so excl_out[d] = d and the call returns GB_OK; 0: nothing publishes
 * tile 0, every wait gives up after spin_limit polls (1 .. 2^20), the
 * call returns GB_ETIMEOUT and *timeouts_out = 256.  Synchronous.  No
 * reference counterpart. */
int gb_sort_wait_probe(int spin_limit, int publish_first, uint32_t *excl_out,
                       uint64_t *timeouts_out);

/* ------------------------------------------------------------ calibration */
/* Launches an FP32 FMA-throughput kernel (packed = 1: .f32x2 form) on
 * `stream`; *flops receives the FLOP count of the launch, which the caller
 * times.  Measures the FP32 CUDA-core peak used as the direct-sum roofline.
 * No reference counterpart (measurement support). */
int gb_calib_fp32(float *scratch, int iters, int packed, double *flops, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GBGRAV_H */
