/*
 * simpimc_gb300 — C interface of the GB300 path-integral Monte Carlo action/estimator library.
 *
 * One context = one simulation (path, actions, moves, observables, algorithm loop) on one GPU,
 * built from a simpimc XML input. Every call returns PIMC_OK (0) or a negative PIMC_ERR_* code;
 * pimc_last_error() gives the message of the last failing call on that context. No call exits
 * the process, traps the device or throws across this boundary.
 *
 * Path buffers crossing the boundary are host arrays in the reference's bead order
 * (species_class.h:236-244, "init_type=File all_beads=1"): pos[g][b][d] with g the particle index
 * over all species in declaration order, b the time slice, d the Cartesian component.
 *
 * Each entry point names the reference interface it replaces (paths inside etano/simpimc).
 */
#ifndef SIMPIMC_GB300_H_
#define SIMPIMC_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PIMC_OK 0
#define PIMC_ERR_ARG (-1)         /* invalid argument (index, range, null pointer) */
#define PIMC_ERR_INPUT (-2)       /* malformed XML, missing attribute or table file */
#define PIMC_ERR_CUDA (-3)        /* CUDA runtime failure */
#define PIMC_ERR_TIMEOUT (-4)     /* a bounded device wait expired */
#define PIMC_ERR_NONFINITE (-5)   /* non-finite coordinate or action difference */
#define PIMC_ERR_UNSUPPORTED (-6) /* input uses a feature outside this library */
#define PIMC_ERR_STATE (-7)       /* call not valid in the current state */

typedef struct pimc_ctx pimc_ctx;

typedef struct pimc_info {
    uint32_t n_d, n_bead, n_species, n_total, n_k, n_actions, n_moves, n_observables;
    double beta, tau, L, volume;
    int32_t pbc;
} pimc_info;

/* Framework + Simulation construction (src/framework/framework_class.h:39-79,
 * src/framework/simulation_class.h:16-39). `base_dir` resolves relative table paths; `chain`
 * selects the independent random stream (the reference's clone index, framework_class.h:104). */
int pimc_create(const char* xml_text, const char* base_dir, int device, uint32_t chain, pimc_ctx** out);
void pimc_destroy(pimc_ctx* ctx);
const char* pimc_last_error(const pimc_ctx* ctx);
int pimc_get_info(pimc_ctx* ctx, pimc_info* out);
/* Overrides the <RNG seed> (framework_class.h:84-101). */
int pimc_set_seed(pimc_ctx* ctx, uint32_t seed);
/* Names: kind 0 species, 1 action, 2 move, 3 observable. */
int pimc_get_name(pimc_ctx* ctx, int kind, uint32_t index, char* buf, size_t cap);
int pimc_species_info(pimc_ctx* ctx, uint32_t species, uint32_t* n_part, uint32_t* offset, double* lambda);

/* Path state: Bead::SetR / StoreR and Species::InitRhoK (bead_class.h:57-101,
 * species_class.h:236-244,380-403). which: 0 the stored ("old") copy, 1 the working ("new") copy,
 * 2 both (then the per-slice charge densities are recomputed from the positions). */
int pimc_set_path(pimc_ctx* ctx, int which, const double* pos);
int pimc_get_path(pimc_ctx* ctx, int which, double* pos);
/* Per-slice charge density of a species, [n_bead][n_k][re, im] (species_class.h:23,428). */
int pimc_get_rho_k(pimc_ctx* ctx, uint32_t species, double* out);
/* Stored half-space k-vectors [n_k][n_d] (k_space_class.h:33-80). */
int pimc_get_kvecs(pimc_ctx* ctx, double* out);

/* Action interface (src/actions/action_class.h:37-52). Particles are (species, index) pairs as
 * in the reference's std::vector<std::pair<std::shared_ptr<Species>, uint32_t>>. mode 0 reads the
 * stored copy (OLD_MODE), 1 the working copy (NEW_MODE, bead_class.h:7-8, 98). */
/* Action::GetAction (action_class.h:43) */
int pimc_get_action(pimc_ctx* ctx, uint32_t action, uint32_t b0, uint32_t b1, const uint32_t* species, const uint32_t* particles,
                    uint32_t n_particles, uint32_t level, int mode, double* out);
/* Same value as pimc_get_action for a pair action, computed without any device allocation
 * during the call: for host programs that give all GPU memory to their own pool or may not
 * allocate where they call from. All temporaries live in one 4 MiB array fixed in the library
 * (held on every GPU that loads it); larger requests fail with PIMC_ERR_ARG. Calls share that
 * array, so calls whose GPU work overlaps race; the first call on a device looks up the array's
 * address and should come before any stream capture. No counterpart in the reference. */
int pimc_get_action_noalloc(pimc_ctx* ctx, uint32_t action, uint32_t b0, uint32_t b1, const uint32_t* species,
                            const uint32_t* particles, uint32_t n_particles, uint32_t level, int mode, double* out);
/* Action::GetActionGradient (action_class.h:46); out has n_d entries. */
int pimc_get_action_gradient(pimc_ctx* ctx, uint32_t action, uint32_t b0, uint32_t b1, const uint32_t* species,
                             const uint32_t* particles, uint32_t n_particles, uint32_t level, int mode, double* out);
/* Exact ("adjoint") counterparts, level 0, FP64. The whole-ring action of one action (action >= 0)
 * or of every action (action = -1): every link b -> b+1 of every particle of its species, the
 * trap on every slice, every pair on every slice and, for Ewald actions, the k-space sum
 * tau sum_b sum_k v_k Re(rho_a conj(rho_b)) (x2 between different species) from densities of the
 * chosen copy. pimc_action_gradient_path returns its gradient dS/dR, grad[p][b][d] in the path
 * order, with the trap and Ewald forces the reference leaves out (pair_action_class.h:305-337,
 * trap_class.h) and the analytic pair derivative in place of its eps = 1e-4 central differences
 * (pair_action_class.h:135-155). pimc_get_action_gradient_exact is Action::GetActionGradient
 * (action_class.h:46) from that gradient: the sum over the listed particles of the action's species
 * and slices b0..b1-1 of dS/dr. No reference counterpart for the first two. */
int pimc_total_action(pimc_ctx* ctx, int action, int mode, double* out);
int pimc_action_gradient_path(pimc_ctx* ctx, int action, int mode, double* grad);
int pimc_get_action_gradient_exact(pimc_ctx* ctx, uint32_t action, uint32_t b0, uint32_t b1, const uint32_t* species,
                                   const uint32_t* particles, uint32_t n_particles, uint32_t level, int mode, double* out);
/* Action::DActionDBeta (action_class.h:37) */
int pimc_dactiondbeta(pimc_ctx* ctx, uint32_t action, double* out);
/* Action::Potential (action_class.h:52) */
int pimc_potential(pimc_ctx* ctx, uint32_t action, double* out);
/* Action::VirialEnergy (action_class.h:40) */
int pimc_virial_energy(pimc_ctx* ctx, uint32_t action, double window, double* out);

/* Moves: Move::DoEvent repeated (move_class.h:61-77, bisect_class.h:24-139). Runs n attempts
 * of move `move` on the device in one launch. Besides Bisect, a <Move type="HMC" step_size="0.01"
 * n_steps="10" [species="..."]/> (no reference counterpart) moves the whole path of one or every
 * species by hybrid Monte Carlo: Gaussian momenta, leapfrog on S(R) + |P|^2/2 with the exact
 * gradient, Metropolis on the energy change. */
int pimc_move_attempts(pimc_ctx* ctx, uint32_t move, uint64_t n);
/* A schedule of moves, (moves[i], counts[i]) in order, repeated n_rep times, in one launch
 * (the body of a Loop of Move events, loop_class.h:55-60). A Bisect move whose Ilkka or David pair
 * action has max_level > 0 runs on the permutation kernel, which forms the pair terms of every
 * level (pair_action_class.h:267-291). A long-range pair action with max_level > 0 in a move of
 * more than one level makes the call fail with PIMC_ERR_UNSUPPORTED before any attempt runs: the
 * reference latches its densities there (pair_action_class.h:293-298). */
int pimc_sweep(pimc_ctx* ctx, const uint32_t* moves, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep);
/* out[5] = {total attempts, attempts in block, accepts in block, total accepts, total attempts
 * that reached the level-0 test} (counters of move_class.h:11-12). */
int pimc_move_stats(pimc_ctx* ctx, uint32_t move, uint64_t* out);

/* Path permutation of a species (the bead links at the ring closure, bead_class.h:38-41 after the
 * relabelling of perm_bisect_class.h:47-56): perm[p] is the particle whose slice-0 bead follows
 * bead (p, M - 1); species-local indices. pimc_set_perm refuses a non-permutation with
 * PIMC_ERR_ARG. Permuting moves (PermBisectIterative, PermBisectTable) and the plain bisection of a
 * species that has one or carries a non-identity permutation run on the permutation kernel. */
int pimc_get_perm(pimc_ctx* ctx, uint32_t species, uint32_t* perm);
int pimc_set_perm(pimc_ctx* ctx, uint32_t species, const uint32_t* perm);
/* pimc_sweep on n_ctx independent chains (contexts of the same input structure on one device):
 * when every schedule entry is a Bisect or permuting move on a species of at most 512 particles,
 * all chains go to one launch of the permutation kernel with one CTA per chain, any action set and
 * either precision included (in 32-bit mode the kernel forms FP32 densities and Ewald terms) (the reference runs one chain per MPI
 * process, framework_class.h:44-53); otherwise the chains run one after another. Errors are
 * reported on ctxs[0]. */
int pimc_sweep_chains(pimc_ctx** ctxs, uint32_t n_ctx, const uint32_t* moves, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep);
/* Per cycle length 1..N of a permuting move: out[0..N) attempts, out[N..2N) accepts of the current
 * block (perm_bisect_class.h:25-26, 59-90); N = the move's species particle count. */
int pimc_perm_stats(pimc_ctx* ctx, uint32_t move, uint64_t* out, size_t cap);

/* Observables: Observable::DoEvent / Write (observable_class.h:93-104). pimc_observable_block
 * returns the normalised values Write() would append (energy_class.h:232-325,
 * pair_correlation_class.h:89-123, structure_factor_class.h:69-85) and resets the block. */
int pimc_observable_accumulate(pimc_ctx* ctx, uint32_t observable);
int pimc_observable_block(pimc_ctx* ctx, uint32_t observable, double* out, size_t cap, size_t* n);

/* Simulation::Run (simulation_class.h:42-45): the XML <Algorithm> loop. Block values are kept
 * per observable and read back with pimc_get_block. */
int pimc_run(pimc_ctx* ctx);
/* The run's output so far (every Write event's move counters and observable blocks, and the path
 * dumps of PathDump observables) under the reference's HDF5 dataset paths (Moves/<name>/...,
 * Observables/<name>/..., Observables/<path dump>/<species>/{n_dump, positions, permutation};
 * move_class.h:45-53, observable_class.h:79-88, path_dump_class.h:28-66), written in the table
 * container format. A species with init_type="Restart" prefix="P" reads the last path dump of
 * P.0.pat (P.<chain>.pat with parallel="1") at creation (species_class.h:336-377). */
int pimc_write_output(pimc_ctx* ctx, const char* path);
int pimc_n_blocks(pimc_ctx* ctx, uint32_t observable, size_t* n);
int pimc_get_block(pimc_ctx* ctx, uint32_t observable, size_t block, double* out, size_t cap, size_t* n);

/* Sweep precision (the reference's build-time PRECISION option, CMakeLists.txt:11-19, as a run-time
 * switch): 64 (default) keeps positions, per-slice densities and all action terms in double-float;
 * 32 keeps the per-slice densities, bead phases and Ewald differences in FP32 with compensated sums
 * (densities rebuilt from the positions at every sweep call, on the sweep kernel and on the
 * permutation kernel alike), while positions, pair links, level sums and the acceptance test stay
 * double-float and estimators stay FP64. */
int pimc_set_precision(pimc_ctx* ctx, int bits);
/* Synchronises the context stream and reports any device-side error (timeout, non-finite). */
int pimc_synchronize(pimc_ctx* ctx);
/* Tuning: CTAs of the cooperative sweep (0 = automatic) and the device wait limit. */
int pimc_set_sweep_grid(pimc_ctx* ctx, int grid);
int pimc_set_timeout_ns(pimc_ctx* ctx, uint64_t ns);
/* Failure-path check of the device wait limit: one wait of the sweep's bounded grid barrier that
 * no block can complete, limited to timeout_ns (at most 10 s). It returns PIMC_ERR_TIMEOUT with
 * the device-measured wait in *waited_ns (may be NULL) and leaves the context usable; the path is
 * not touched. When a real launch times out, its blocks may have committed parts of an attempt:
 * every call that reads or moves the path then returns PIMC_ERR_STATE until
 * pimc_set_path(ctx, 2, ...). The reference has no counterpart (its errors exit the process,
 * actions.h:32-33). */
int pimc_check_wait_limit(pimc_ctx* ctx, uint64_t timeout_ns, uint64_t* waited_ns);
/* Bisection attempts in flight per round of the sweep (1..8; 0, the default, = automatic): the
 * blocks split into that many groups, and each round runs the longest prefix of the schedule's next
 * attempts in which no attempt reads what an earlier one may change (no earlier attempt's inner
 * slices meet its closed segment). The Markov chain is the sequential one, bit for bit. Automatic
 * takes 2 when a segment's density work (2^max_level slices x k-vectors) is at most 2^17 and 1
 * otherwise. Schedules with a move that has no pair action, or a segment longer than half the
 * ring, run one attempt at a time. */
int pimc_set_sweep_wave(pimc_ctx* ctx, int wave);
/* CUDA stream of the context (cudaStream_t), for callers that enqueue their own work. */
void* pimc_stream(pimc_ctx* ctx);
/* Sweep tracing, the device-side analogue of the reference's per-event timers (move_class.h:61-77,
 * time_class.h:38-68): cycles spent by block 0 in the 8 phases of each attempt (segment and random
 * numbers, sampling, per-level terms, grid work, grid barrier, final sum, decision, commit),
 * followed by the slowest warp of each of 8 roles inside phases 2-4 (sampling chain, stored-copy
 * level sums, old phase tables, stored-copy pair links, working-copy level sums, new phase tables,
 * old Ewald phases, grid-phase pair links and Ewald cells). `cycles` (16 entries, may be NULL)
 * receives the sums since the last reset; `enable` >= 0 switches recording on/off and resets the
 * sums (-1 leaves both as they are). */
int pimc_sweep_timing(pimc_ctx* ctx, int enable, uint64_t* cycles);

/* ---------------------------------------------------------------------------------------------
 * Batched independent chains. The reference obtains several Markov chains only as MPI clones,
 * one process each with its own seed, input and output (framework_class.h:44-53,84-99); this
 * handle runs many chains, one XML input each, in one persistent launch per call. Chain i draws
 * from the same counter-based stream as a single-chain context created with chain = i, so it
 * replays that context's Markov chain up to FP32 rounding (positions and per-term actions in
 * FP32, sums in double-float, estimator values in FP64).
 * Supported inputs: one 3-D species, Kinetic (n_images 0), optional HarmonicTrap, optional
 * BarePairAction is_coulomb=1 without long range within the species, one fixed-level Bisect with
 * n_level <= 5; anything else returns PIMC_ERR_UNSUPPORTED. */
typedef struct pimc_batch pimc_batch;

int pimc_batch_create(const char* const* xml_texts, uint32_t n_chains, const char* base_dir, int device, pimc_batch** out);
void pimc_batch_destroy(pimc_batch* b);
const char* pimc_batch_last_error(const pimc_batch* b); /* NULL handle: last failed create */
/* out4 = {n_part, n_bead, n_level, warps of its pair tile}. */
int pimc_batch_chain_info(pimc_batch* b, uint32_t chain, uint32_t* out4);
/* One chain's path, pos[p][b][d] as for pimc_set_path (stored as FP32). */
int pimc_batch_set_path(pimc_batch* b, uint32_t chain, const double* pos);
int pimc_batch_get_path(pimc_batch* b, uint32_t chain, double* pos);
/* Every chain's path in one transfer: the chains' [n_part][n_bead][3] arrays concatenated in chain
 * order, copied as they are (one copy each way; pinned host memory moves at full link speed) and
 * laid out on the device. A non-finite coordinate makes set_paths return PIMC_ERR_ARG. */
int pimc_batch_set_paths(pimc_batch* b, const double* all);
int pimc_batch_get_paths(pimc_batch* b, double* all);
/* n bisection attempts (Move::DoEvent, move_class.h:61-77) on every chain. */
int pimc_batch_attempts(pimc_batch* b, uint64_t n);
/* n sweeps on every chain; a sweep of a chain is n_part * ceil(n_bead / 2^n_level) attempts. */
int pimc_batch_sweeps(pimc_batch* b, uint64_t n);
/* One thermal energy measurement on every chain (Energy::Accumulate, energy_class.h:36-58). */
int pimc_batch_measure(pimc_batch* b);
/* n_cycles replays of a CUDA graph holding `sweeps_per_measure` sweeps and one measurement. */
int pimc_batch_run(pimc_batch* b, uint64_t n_cycles, uint64_t sweeps_per_measure);
int pimc_batch_sync(pimc_batch* b);
/* Energy series of one chain: out[m][4] = {E, kinetic, trap, pair} per measurement, each already
 * divided by n_bead as in Energy::Write (energy_class.h:232-253); at most `cap` rows (the device
 * keeps the first 4096); *n_measure = measurements since the last reset. */
int pimc_batch_energy(pimc_batch* b, uint32_t chain, double* out, uint64_t cap, uint64_t* n_measure);
int pimc_batch_reset_energy(pimc_batch* b);
/* The latest measurement of every chain, out[n_chains][4] = {E, kinetic, trap, pair}. */
int pimc_batch_last_energy(pimc_batch* b, double* out);
/* Per-chain attempt and acceptance counters (arrays of n_chains; either may be NULL). */
int pimc_batch_counters(pimc_batch* b, uint64_t* attempts, uint64_t* accepts);
/* Scheduling rounds of the bisection sweep kernel per chain (array of n_chains) since creation: a
 * round runs up to `wave` commuting attempts of the chain at once, so attempts / rounds is the
 * chain's concurrency and the heaviest chain's rounds set the sweep launch's critical path. No
 * reference counterpart (a diagnostic of this library's scheduler). */
int pimc_batch_rounds(pimc_batch* b, uint64_t* rounds);
/* Split chains: the n most expensive chains whose tile uses 16 warps with a wave and a path staged in
 * shared memory each run on a cluster of two blocks (four groups of four warps per block, both
 * blocks holding the path and the same scheduler; a round runs up to eight commuting attempts and
 * every commit is written into both blocks' copies); the other chains pair up, two per cluster. The
 * Markov chains are unchanged. pimc_batch_get_split returns how many chains qualified and were
 * split (0: the plain one-block-per-chain launch); pimc_batch_autotune tries 0, 8, 16 and 32. */
int pimc_batch_set_split(pimc_batch* b, uint32_t n);
int pimc_batch_get_split(pimc_batch* b, uint32_t* n);
/* Overlapped measurement cycle: with heavy = H > 0 and HMC attempts in the cycle, pimc_batch_run's
 * graph runs the H most expensive chains' sweeps and HMC attempts on one stream and the other
 * chains' on a second stream at the same time (each chain's kernels in order, then one energy
 * measurement of every chain), so the lighter chains' HMC fills the SMs their sweeps leave while the
 * heavy sweeps finish. The Markov chains are unchanged; pimc_batch_autotune tries H = 0, n/8, n/4,
 * 3n/8, n/2 and 5n/8 of the n chains (0: one stream), timing each by the median of five cycles. */
int pimc_batch_set_overlap(pimc_batch* b, uint32_t heavy);
int pimc_batch_get_overlap(pimc_batch* b, uint32_t* heavy);
/* Hybrid Monte Carlo on the batch ("batched + adjoint"; no reference counterpart): a chain's input
 * may hold one <Move type="HMC" step_size="..." n_steps="..."/> besides its Bisect move. Each
 * attempt draws Gaussian momenta for every bead from the move's stream (keyed by its index in the
 * input, as in a single-chain context), runs the leapfrog on S(R) + |P|^2/2 with the exact gradient
 * of the whole-ring kinetic, trap and bare Coulomb action (pimc_action_gradient_path), and accepts
 * with probability min(1, exp(-dH)). Positions, momenta and forces are FP32; both energies are
 * double-float sums of exact differences and dH is FP64. Each chain runs on a thread-block cluster
 * of k = 1, 2, 4 or 8 blocks (one k for the launch; it must divide every HMC chain's n_bead): block r
 * holds slices [r n_bead / k, (r + 1) n_bead / k) with one halo slice on each side and their momenta
 * in shared memory, 24 n_part (n_bead / k + 1) bytes, and reads the halos from its neighbours'
 * shared memory after every drift. The trajectory does not depend on k (every bead's force and
 * update is the same FP32 sequence); the energies' last bits may. pimc_batch_hmc_attempts runs n
 * attempts on every chain with the move;
 * pimc_batch_hmc_counters reads their attempt and accept counters; pimc_batch_set_hmc_per_cycle adds
 * n attempts to every measurement cycle of pimc_batch_run (after the sweeps);
 * pimc_batch_set_hmc_cluster / pimc_batch_get_hmc_cluster set and read k (pimc_batch_autotune picks
 * the fastest that fits; error kErrUnsupported where k does not divide an n_bead or does not fit). */
int pimc_batch_hmc_attempts(pimc_batch* b, uint64_t n);
int pimc_batch_hmc_counters(pimc_batch* b, uint64_t* attempts, uint64_t* accepts);
int pimc_batch_set_hmc_per_cycle(pimc_batch* b, uint64_t n);
int pimc_batch_set_hmc_cluster(pimc_batch* b, uint32_t k);
int pimc_batch_get_hmc_cluster(pimc_batch* b, uint32_t* k);
/* Tiles: one attempt wants ceil((n_part-1)(2^n_level-1) / (32 items_per_lane)) warps for its pair
 * items; with wave = 1 a chain gets that many, at most max_warps (<= 16). With wave = W > 1 (<= 8)
 * a chain runs up to W attempts at once on W groups of such warps (at least 2 each, W times at
 * most max_warps in all): of its next 32 drawn attempts, the first W that commute with every
 * earlier attempt not yet run (neither reads what the other writes), possibly out of order, so the
 * Markov chain is the sequential one. pimc_batch_autotune times `trial_sweeps` sweeps of every
 * candidate (and the split-chain counts, HMC cluster sizes and overlapped cycles) on a saved copy of
 * the chains' state, restores it, and keeps the fastest. */
int pimc_batch_set_tiles(pimc_batch* b, uint32_t items_per_lane, uint32_t max_warps, uint32_t wave);
int pimc_batch_autotune(pimc_batch* b, uint32_t trial_sweeps, uint32_t* items_per_lane, uint32_t* max_warps, uint32_t* wave,
                        double* sec_per_sweep);
/* out4 = {n_chains, bead moves per sweep of all chains, kernels launched so far, series rows kept}. */
int pimc_batch_stats(pimc_batch* b, uint64_t* out4);
/* CUDA stream of the batch (cudaStream_t). */
int pimc_batch_stream(pimc_batch* b, void** stream);

#ifdef __cplusplus
}
#endif

#endif /* SIMPIMC_GB300_H_ */
