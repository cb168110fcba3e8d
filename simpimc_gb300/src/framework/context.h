// Host-side owner of one simulation on one GPU: the counterpart of the reference's Simulation
// (src/framework/simulation_class.h:8-46), which owns the Path, the actions, the moves and the
// observables. Here the path, tables and accumulators live in device memory and every
// action/move/observable call launches a kernel on the context's stream.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../data_structures/system.h"
#include "input.h"

namespace pimc {

struct PimcError : std::runtime_error {
    int code;
    PimcError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Status codes returned through the C interface (mirrored in include/simpimc_gb300.h).
enum : int {
    kOk = 0,
    kErrArg = -1,
    kErrInput = -2,
    kErrCuda = -3,
    kErrTimeout = -4,
    kErrNonFinite = -5,
    kErrUnsupported = -6,
    kErrState = -7,
};

void CudaCheck(cudaError_t e, const char* what);
/// Loads the FP64 conversion kernels of the sweep (EnsureFP64) ahead of their first launch.
void PreloadConversionKernels();

/// Owning device allocation.
struct DeviceBuffer {
    void* ptr = nullptr;
    size_t bytes = 0;
    DeviceBuffer() = default;
    explicit DeviceBuffer(size_t n);
    ~DeviceBuffer();
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    template <class T>
    T* as() const { return static_cast<T*>(ptr); }
};

struct ActionHost {
    std::string name, type;
    int kind = 0;   // 0 kinetic, 1 trap, 2 bare pair
    int index = 0;  // into SystemDev::{kinetic,trap,pair}
    std::vector<uint32_t> species_list;
    bool is_importance_weight = false;
    // PairAction::is_first_time / dUdB_constant / potential_constant (pair_action_class.h:14-19)
    bool is_first_time = true;
    double dUdB_constant = 0., potential_constant = 0.;
};

struct MoveHost {
    std::string name, type;
    MoveDev dev;
    bool adaptive = false;
    double target_ratio = 0.;
    bool first_block = true;
    uint64_t attempts = 0;       // total attempts (Philox attempt counter)
    uint64_t block_attempt = 0;  // counters since the last Write (move_class.h:37-40)
    uint64_t block_accept = 0;
    double last_ratio = 0.;      // acceptance ratio of the last completed block
    uint64_t total_accept = 0;   // accepted attempts since construction
    uint64_t total_level0 = 0;   // attempts whose proposal reached the level-0 evaluation
    // Per Write event (move_class.h:80-94, bisect_class.h:193-213): the block's counters, its
    // acceptance ratio and the bisection level in force.
    std::vector<double> out_attempt, out_accept, out_ratio, out_level;
    // Hybrid Monte Carlo move (no reference counterpart): leapfrog on the whole path driven by
    // the adjoint gradient of the total action.
    int kind = 0;                // 0 Bisect, 1 HMC, 2 PermBisectIterative, 3 PermBisectTable
    // Permuting bisection (perm_bisect_class.h:19-29): epsilon of the weight table, per cycle
    // length the block's attempts and accepts (appended per Write), and for the table variant the
    // particle subsets and their permutations (lexicographic order) on the device.
    double perm_epsilon = 1.e-100;
    uint32_t perm_k = 0, perm_n_comb = 0, perm_n_types = 0, perm_n_type_out = 0;
    std::vector<uint64_t> perm_attempt, perm_accept;
    std::vector<std::vector<double>> out_perm_attempt, out_perm_accept;
    std::shared_ptr<DeviceBuffer> perm_combs, perm_types;
    double hmc_step = 0.01;
    uint32_t hmc_steps = 10;
    int hmc_species = -1;        // -1: every species moves
};

struct ObservableHost {
    std::string name, type;
    int kind = 0;  // 0 energy, 1 pair correlation, 2 structure factor, 3 ignored bookkeeping, 4 path dump,
                   // 5 sign, 6 permutation
    uint64_t n_measure = 0;
    // Energy (energy_class.h:7-326)
    bool measure_potential = false, use_thermal = true, use_virial = false;
    bool use_adjoint = false;  // virial centroid from the adjoint gradient of every non-kinetic action
    uint32_t virial_window = 0;
    std::vector<double> energies, potentials;
    // PairCorrelation (pair_correlation_class.h:7-124)
    uint32_t sa = 0, sb = 0, n_r = 0;
    double r_min = 0., r_max = 0., dr = 0., d_ir = 0.;
    std::unique_ptr<DeviceBuffer> hist;  // unsigned long long [n_r]
    // StructureFactor (structure_factor_class.h:7-86)
    double k_cut = 0.;
    std::unique_ptr<DeviceBuffer> sk;    // double [K]
    // PathDump (path_dump_class.h:7-70): every `skip`-th Write stores each species' positions as
    // the reference's cube (n_d, n_bead, n_part), column-major, and its permutation (2, n_part).
    uint32_t skip = 1;
    uint64_t n_write_calls = 0;
    std::vector<std::vector<std::vector<double>>> dumps;  // [species][dump] positions
    std::vector<std::vector<std::vector<double>>> dump_perms;  // [species][dump] (prev, next) per particle
    // Sign (sign_class.h:7-48) and Permutation (permutation_class.h:7-119): the block's sign sum,
    // cycle-length counts and sector of each measurement; the partitions of N in sector order.
    double sign_sum = 0.;
    uint32_t species = 0, sector_max = 0;
    std::vector<double> cycles;
    std::vector<uint32_t> sectors;
    std::vector<std::vector<uint32_t>> partitions;
};

struct LoopNode {
    int kind = 0;  // 0 loop, 1 move, 2 observable, 3 write
    uint32_t index = 0;
    uint64_t n_steps = 1;
    std::vector<LoopNode> children;
};

class Context {
   public:
    Context(const Input& in, const std::string& base_dir, int device, uint32_t chain);
    ~Context();

    // --- path state (path_class.h / species_class.h) ---
    void SetPath(int which, const double* host_pos);  // [n_total][M][n_d]; which 0 old, 1 new, 2 both
    void GetPath(int which, double* host_pos);
    void InitRhoK();                                   // species_class.h:380-403 for every kept species
    void ComputeRho(const double* pos, double2* out);  // the same densities of any position copy into `out`
    void GetRhoK(uint32_t species, double* out);       // [M][K][2]
    void GetKVecs(double* out);                        // [K][n_d]

    // --- Action interface (action_class.h:37-52) ---
    double GetAction(uint32_t a, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n, uint32_t level, int mode);
    void GetActionGradient(uint32_t a, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n, uint32_t level,
                           int mode, double* out);
    double DActionDBeta(uint32_t a);
    double Potential(uint32_t a);
    double VirialEnergy(uint32_t a, double window);
    double VirialCentroid(uint32_t species);  // centroid term of energy_class.h:78-94 (before / 2 tau)

    // --- adjoint: the whole-ring action at level 0 and its exact gradient dS/dR ---
    double TotalAction(int a, int mode);                          // action a, or every action for a = -1
    void ActionGradientPath(int a, int mode, double* host_grad);  // [n_total][M][n_d]
    void ActionGradientAdjoint(uint32_t a, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n,
                               uint32_t level, int mode, double* out);
    double VirialCentroidAdjoint(uint32_t species);
    void HmcAttempts(uint32_t m, uint64_t n);
    // Device-side pieces (a >= 0 one action, -1 every action, -2 every non-kinetic action).
    double TotalActionDev(int a, const double* pos, const float4* rho);
    void GradientDev(int a, const double* pos, const float4* rho, double* grad);  // [M][3][n_pad], overwritten
    const float4* ScratchRho(const double* pos);                                    // double-float densities of `pos`

    // --- moves, observables, algorithm ---
    void MoveAttempts(uint32_t m, uint64_t n);
    // Bisection on a species with exchanges (src/kernels/perm.cu): the permuting moves and the
    // plain bisection of a species that has one or carries a non-identity path permutation.
    void PermAttempts(uint32_t m, uint64_t n);
    void PermEnqueue(uint32_t m, uint64_t n);
    void PermFinish();
    void PermPrepare(const uint32_t* mv, uint32_t n_entries);
    void PermDensities();  // FP32 mode: FP32 densities from the positions before permutation-kernel launches
    void PermArgs(uint32_t m, void* out, size_t* smem);  // the kernel's arguments for move m (sweep.cu)
    uint32_t perm_pending_ = 0;  // moves with permutation launches not yet folded into their counters
    void* MoveDescriptors();  // double-float move descriptors on the device (sweep.cu)
    bool PermutingSpecies(uint32_t s) const;
    bool LevelPairTerms(uint32_t m) const;  // Bisect move with pair terms above level 0 (sweep.cu)
    void RequireLevelZeroDensities(uint32_t m) const;  // refuses Ewald parts above level 0 (sweep.cu)
    // The path permutation: perm[g] = particle whose slice-0 bead follows bead (g, M - 1), global
    // indices; the host copy is refreshed after every device update.
    void SyncPermHost();
    bool PermIdentity(uint32_t s) const;
    bool AnyPerm() const;
    void SetPerm(uint32_t s, const uint32_t* pi);  // species-local indices
    void GetPerm(uint32_t s, uint32_t* out) const;
    std::vector<uint32_t> CycleLengths(uint32_t s) const;
    double PathSign() const;
    std::vector<uint32_t> perm_host;
    std::vector<int> species_fermi;
    void Sweep(const uint32_t* moves, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep);
    void ObservableAccumulate(uint32_t o);
    std::vector<double> ObservableBlock(uint32_t o);
    void Run();
    void RunNode(const LoopNode& n);
    void WriteBlock();

    // --- configuration ---
    SystemDev sys;
    int device = 0;
    int n_sm = 0;
    cudaStream_t stream = nullptr;
    uint32_t seed = 12345, chain = 0;
    uint64_t timeout_ns = 2000000000ull;
    int sweep_grid = 0;       // CTAs of the cooperative sweep (0 = automatic)
    int sweep_wave = 0;       // bisection attempts in flight per round of the sweep (0 = automatic)
    int last_grid_ = 0;       // CTAs of the most recent sweep launch
    bool phase_timing = false;  // record per-phase cycles of block 0 in the sweep kernel
    std::unique_ptr<DeviceBuffer> phase_buf;  // unsigned long long [kSweepPhases]
    std::vector<std::string> species_names;
    // Species initialised from a previous run's path dump (species_class.h:336-377).
    struct RestartSpec {
        uint32_t species;
        std::string file, dump_name;
    };
    std::vector<RestartSpec> restarts;
    void ApplyRestarts();
    /// The run's output under the reference's dataset paths (Moves/*, Observables/*) in the table
    /// container format.
    void WriteOutput(const std::string& path);
    std::vector<ActionHost> actions;
    std::vector<MoveHost> moves;
    std::vector<ObservableHost> observables;
    LoopNode main_loop;
    std::vector<std::vector<std::vector<double>>> blocks;  // per observable, per block
    std::vector<double> kmags;                             // |k| per stored k-vector
    double kcutoff = 0.;                                   // KSpace::cutoff after all setups
    std::vector<std::vector<int>> kint;                    // integer k indices per stored k-vector
    int rho_slots = 0;
    std::string base_dir;

    // Double-float mirrors of the path state used by the sweep kernel (positions as (hi, lo)
    // float pairs, per-slice densities as (re.hi, re.lo, im.hi, im.lo)). Exactly one of the two
    // representations may be newer than the other; Ensure* converts on demand.
    void EnsureDD();
    void EnsureFP64();
    // Sweep precision: 64 keeps the densities in double-float; 32 keeps them (and the bead phases
    // and Ewald differences) in FP32 with compensated sums, rebuilt from the positions per call.
    void SetPrecision(int bits);
    int precision = 64;
    bool dd_valid = false;
    bool fp64_valid = true;
    // Host copies of every spline table, keyed by the device coefficient pointer, so the sweep
    // can build double-float versions of the same tables.
    struct HostCubic {
        std::vector<double> x;
        std::vector<Cubic4> c;
        std::vector<int32_t> bucket;
    };
    std::vector<std::pair<const Cubic4*, HostCubic>> host_cubics;
    struct HostBicubic {
        std::vector<double> x, y;
        std::vector<double> c;  // [cells][16]
        std::vector<int32_t> bx, by;
    };
    std::vector<std::pair<const double*, HostBicubic>> host_bicubics;
    struct HostMulti {
        std::vector<double> x;
        std::vector<Cubic4> c;  // [interval][component]
        std::vector<int32_t> bucket;
        int32_t n_comp;
    };
    std::vector<std::pair<const Cubic4*, HostMulti>> host_multis;
    // Per pair action, the k-space coefficient of its long-range action: v_long_k for the bare action
    // (multiplied by tau 2^level there), u_long_k / tau for IlkkaPairAction (empty without long range).
    std::vector<std::vector<double>> host_vk;

   private:
    std::vector<std::unique_ptr<DeviceBuffer>> keep_;  // tables owned for the context lifetime
    std::unique_ptr<DeviceBuffer> pos_dd_, rho_dd_, rho32_, sweep_desc_, sweep_tables_, sched_wave_;
    bool sweep_tables_built_ = false;
    std::vector<uint32_t> desc_levels_;  // bisection levels the uploaded move descriptors were built for
    struct StageTable {
        const void* x;  // float2 knots
        const void* c;  // float4 coefficients
        uint32_t n;
    };
    std::vector<StageTable> stage_tables_;  // spline tables the sweep may copy into shared memory
    void BuildSweepTables();
    void PairGradDD(uint32_t pair, const double* pos, double* grad);  // double-float short-range pair forces (sweep.cu)
    std::unique_ptr<DeviceBuffer> pos_, pos_new_, rho_, kidx_;
    std::unique_ptr<DeviceBuffer> grad_, mom_, pos_save_, rho_scratch_, phase_tab_;  // adjoint / HMC work arrays
    std::vector<std::unique_ptr<DeviceBuffer>> adj_vk_;                              // double-float v_k per action
    std::unique_ptr<DeviceBuffer> ewald_w_, ewald_terms_;  // per-species Ewald weight W_s; its terms (v_k pointers, slots)
    std::unique_ptr<DeviceBuffer> partials_, result_, bar_, err_, pairs_, rho_tmp_, parts_, kmag_dev_, sched_, accepts_;
    std::unique_ptr<DeviceBuffer> perm_, perm_inv_, perm_t_, perm_cyc_, perm_drho_, perm_hold_, perm_cnt_, perm_prop_, perm_segold_;
    size_t partials_cap_ = 0, pairs_cap_ = 0, rho_tmp_cap_ = 0, parts_cap_ = 0;

    template <class T>
    T* Upload(const std::vector<T>& v);
    void BuildPath(const Input& in);
    void BuildActions(const Input& in);
    void BuildMoves(const Input& in);
    void BuildObservables(const Input& in);
    void ReadLoop(const Input& in, LoopNode& node);
    CubicTable BuildCubic(const std::vector<double>& x, const std::vector<double>& y, bool uniform);
    BicubicTable BuildBicubic(const std::vector<double>& x, const std::vector<double>& y, const std::vector<double>& f);
    MultiCubic BuildMultiCubic(const std::vector<double>& x, const std::vector<std::vector<double>>& comps);
    void FreeSplineTable(double L, uint32_t n_images, double lambda, double tau, bool want_dtau, CubicTable* image, CubicTable* dtau);

   public:
    // scratch helpers used by the kernel launch wrappers
    double* Partials(size_t n);
    double* Result() { return result_->as<double>(); }
    unsigned long long* Barrier() { return bar_->as<unsigned long long>(); }
    int* ErrWord() { return err_->as<int>(); }
    uint32_t* Pairs(size_t n_pairs);
    double2* RhoTmp(size_t n);
    uint32_t* Parts(size_t n);
    /// Reads and clears the device error word; a timeout of a launch that writes the path marks the
    /// path as lost (path_lost) until the next pimc_set_path(ctx, 2, ...).
    void CheckDeviceError(bool path_written = true);
    void RequirePath() const;  // throws PIMC_ERR_STATE while path_lost
    bool path_lost = false;
    /// One bounded device wait that no block can complete (the sweep's grid barrier at a generation
    /// nobody reaches); returns the device-measured wait and throws PIMC_ERR_TIMEOUT as a sweep would.
    void CheckWaitLimit(uint64_t timeout_ns, uint64_t* waited_ns);
    void Sync();
};

/// The same move schedule (pimc_sweep) on many independent chains, one context each, on one
/// device: schedules that run on the permutation kernel go to one launch with one CTA per chain;
/// others run chain after chain.
void SweepChains(const std::vector<Context*>& cs, const uint32_t* mv, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep);

}  // namespace pimc
