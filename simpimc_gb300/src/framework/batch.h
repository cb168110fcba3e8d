// Many independent Markov chains advanced together on one GPU.
//
// The reference runs one chain per process and gets more chains from MPI clones, each with its
// own seed and output (src/framework/framework_class.h:44-53,84-99). Here the chains are the
// batch dimension of one persistent launch: thread block c runs chain order[c], with as many
// warps as that chain's pair tile needs; chains may differ in particle number, slice number,
// bisection level and seed. A measurement cycle (sweeps, then one energy measurement per chain)
// is captured once as a CUDA graph and replayed; the per-chain attempt counters and estimator
// series live in device memory, so replays advance the chains without host work.
//
// Supported chains (anything else is rejected at creation): one species in three dimensions;
// Kinetic (n_images 0); optional HarmonicTrap; optional BarePairAction with is_coulomb=1 and no
// long-range part between the species and itself; one non-adaptive Bisect move with n_level <= 5
// and optionally one HMC move of the species (the library's whole-path hybrid Monte Carlo move);
// open or periodic boundaries.
//
// Arithmetic: positions and per-term action values in FP32; every sum of terms compensated
// (cascaded TwoSum, as accurate as a sum in twice the working precision); the per-level
// acceptance accumulation (sampling ratio minus this level's action change plus the previous
// level's) and its comparison with the log-uniform draw in double-float (FP32 pairs, 48-bit
// significand): each FP64 instruction holds GB300's FP64 pipe (2 lanes per SM per clock) for a
// whole warp, and the double-float result is within 1e-13 of the FP64 one. Estimator values and
// block sums are FP64.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "context.h"

namespace pimc {

constexpr uint32_t kBatchMaxLevels = 5;        // segment of at most 32 beads
constexpr uint32_t kBatchMaxWarps = 16;        // warps per chain (block size 512)
constexpr uint32_t kBatchSeriesComponents = 4; // E, kinetic, trap, pair (each / M)
constexpr uint32_t kMaxWave = 8;               // attempts of one chain in flight at once

/// Per-chain parameters read by the batched kernels.
struct ChainDev {
    uint32_t n_part, n_bead, n_pad, n_level;  // B = 2^n_level beads per segment
    uint32_t seed, chain_id, n_warps, move;   // Philox keys; warps used; move index in its input
    uint32_t n_wave, sub_warps, staged, pad3; // attempts in flight per round; warps per attempt;
                                              // path held in shared memory during a sweep
    uint64_t pos_off;                         // first float4 of the chain's [n_bead][n_pad] block
    uint64_t attempts_per_sweep;              // n_part * ceil(n_bead / B)
    float L, iL, lambda, tau;
    float sigma[kBatchMaxLevels];        // sqrt(lambda tau 2^l): sampling width at level l
    float i4lt_sample[kBatchMaxLevels];  // 1/(4 lambda (tau 2^l / 2)): sampling density at level l
    float i4lt_level[kBatchMaxLevels];   // 1/(4 lambda tau 2^l): kinetic action at level l
    int32_t pbc, has_trap, has_pair, trap_max_level;
    float trap_cofa, r2_min, r2_max, pad1;  // pair clamp r in [r_min, r_max] as r^2
    double trap_cofb, kin_const, i4ltt;     // DActionDBeta constants (trap_class.h, kinetic_class.h)
    float hmc_eps;                          // HMC leapfrog step (0: the chain has no HMC move)
    uint32_t hmc_steps, hmc_move, pad4;     // leapfrog steps; the HMC move's index in its input
};

/// Host view of one chain's input.
struct ChainSpec {
    uint32_t n_part = 0, n_bead = 0, n_level = 0, seed = 0, move = 0;
    bool has_hmc = false;             // a <Move type="HMC"> besides the Bisect move
    uint32_t hmc_move = 0, hmc_steps = 0;
    double hmc_eps = 0.;
    double beta = 0., tau = 0., L = 0., lambda = 0., omega = 0., r_min = 0., r_max = 0.;
    bool pbc = true, has_trap = false, has_pair = false;
    uint32_t trap_max_level = 0;
};

/// Parses one chain's XML input (the reference's format) into a ChainSpec; throws PimcError
/// (kErrUnsupported) for inputs outside the supported subset.
ChainSpec ParseChain(const std::string& xml, const std::string& base_dir);

class ChainBatch {
   public:
    ChainBatch(const std::vector<std::string>& xml, const std::string& base_dir, int device);
    ~ChainBatch();
    ChainBatch(const ChainBatch&) = delete;
    ChainBatch& operator=(const ChainBatch&) = delete;

    void SetPath(uint32_t chain, const double* pos);  // [n_part][n_bead][3]
    void GetPath(uint32_t chain, double* pos);
    void SetPaths(const double* all);  // every chain's path, concatenated in chain order
    void GetPaths(double* all);
    void LastEnergy(double* out);      // [n_chains][4]: the latest measurement of every chain
    void Attempts(uint64_t n);                // n bisection attempts on every chain
    void HmcAttempts(uint64_t n);             // n HMC attempts on every chain that has the move
    void ReadHmcCounters(uint64_t* attempts, uint64_t* accepts);
    void SetHmcPerCycle(uint64_t n);          // HMC attempts in each graph-replayed cycle
    void SetHmcCluster(uint32_t k);           // thread blocks per chain in the HMC launch (1, 2, 4, 8)
    size_t HmcSmem(uint32_t k) const;         // dynamic shared memory of one HMC block; 0 if k is invalid
    void Sweeps(uint64_t n);                  // n sweeps on every chain (one launch)
    void Measure();                           // one energy measurement on every chain
    void Run(uint64_t n_cycles, uint64_t sweeps_per_measure);  // graph-replayed cycles
    uint64_t ReadEnergy(uint32_t chain, double* out, uint64_t cap);  // series [n][4]
    void ResetEnergy();
    void ReadCounters(uint64_t* attempts, uint64_t* accepts);
    void ReadRounds(uint64_t* rounds);        // scheduling rounds of the sweep kernel per chain
    void SetTiles(uint32_t items_per_lane, uint32_t max_warps, uint32_t wave);
    void SetSplit(uint32_t n);                // the n most expensive chains on two blocks each
    double Autotune(uint32_t trial_sweeps);   // returns the best trial's seconds per sweep (also picks hmc_cluster)
    void Sync();

    uint32_t n_chains = 0, series_cap = 0;
    int device = 0, n_sm = 0;
    uint32_t items_per_lane = 2, max_warps = 16, wave = 1;  // pair tile and attempts in flight per chain
    uint32_t split_request = 0;       // chains asked to run on two-block clusters
    uint32_t overlap_heavy = 0;       // cycle graph: the heaviest chains' sweep beside the others' sweep and HMC
    uint32_t n_split_ = 0, n_clusters_ = 0;  // chains split, clusters of the launch (0: plain launch)
    cudaStream_t stream = nullptr;
    std::vector<ChainSpec> specs;
    std::vector<ChainDev> chains;
    std::vector<uint32_t> order;   // block -> chain, most expensive first
    uint64_t bead_moves_per_sweep = 0;
    uint64_t bead_moves_per_hmc = 0;  // beads one HMC attempt of every chain moves (n_part n_bead each)
    uint64_t hmc_per_cycle = 0;
    uint32_t hmc_cluster = 1;         // thread blocks (one cluster) per chain in the HMC launch
    size_t hmc_smem_cap = 0;          // dynamic shared memory a block of the HMC launch may take
    uint64_t path_doubles = 0;  // sum of n_part * n_bead * 3 over the chains
    uint64_t kernel_launches = 0;
    size_t stage_cap = 0;     // shared memory a sweep block may take for a staged path
    size_t stage_bytes = 0;   // shared memory the sweep launch requests (largest staged path)

   private:
    void Upload();
    // chains order[first .. first + count) on stream s (the batch's stream when null)
    void LaunchSweep(uint64_t n_sweeps, uint64_t n_attempts, uint32_t first = 0, uint32_t count = 0xffffffffu, cudaStream_t s = nullptr);
    void ApplySplit();
    void LaunchHmc(uint64_t n_attempts, uint32_t first = 0, uint32_t count = 0xffffffffu, cudaStream_t s = nullptr);
    void LaunchMeasure(uint32_t i0 = 0, uint32_t i1 = 0xffffffffu, cudaStream_t s = nullptr);  // chains order[i0 .. i1)
    void ResetGraph();
    std::unique_ptr<DeviceBuffer> pos_, chains_dev_, order_dev_, att_, acc_, series_, n_meas_, err_, last_, rounds_;
    std::unique_ptr<DeviceBuffer> hmc_att_, hmc_acc_;  // HMC counters per chain
    std::unique_ptr<DeviceBuffer> cluster_tasks_;      // uint2 per cluster of the split launch
    std::vector<uint2> cluster_tasks_host_;
    bool HmcClusterFits(uint32_t k) const;
    std::vector<uint64_t> path_off_;  // first double of each chain in the concatenated host layout
    std::unique_ptr<DeviceBuffer> dstage_, path_off_dev_;  // host-layout doubles on the device, offsets
    size_t pos_float4 = 0;
    cudaGraphExec_t graph_ = nullptr;
    uint64_t graph_sweeps_ = 0, graph_hmc_ = 0;
    uint32_t graph_heavy_ = 0;
    cudaStream_t side_ = nullptr;                      // second stream of the overlapped cycle
    cudaEvent_t ev_fork_ = nullptr, ev_join_ = nullptr;
    uint32_t launches_per_cycle_ = 3;  // sweep + energy parts + energy finish
    std::unique_ptr<DeviceBuffer> energy_tasks_, energy_first_, energy_part_;
    uint32_t n_energy_tasks_ = 0;
    std::vector<uint32_t> energy_first_host_;  // first energy task of each order position (n_chains + 1)
    size_t energy_smem_ = 0;  // dynamic shared memory of the energy kernel
};

}  // namespace pimc
