// Device-side description of one path-integral system: structure-of-arrays path layout, k-space,
// spline tables and the action/move parameters the kernels read.
//
// Replaces the reference's pointer-linked object graph (Path -> Species -> Bead with per-bead
// std::shared_ptr links and Armadillo vectors, src/data_structures/path_class.h:7-196,
// species_class.h:7-446, bead_class.h:11-149) by flat arrays in HBM:
//
//   pos   [M][3][n_pad]  double   bead positions, slice-major, one row per Cartesian component,
//                                  all species' particles concatenated (species s occupies
//                                  [sp_off[s], sp_off[s] + sp_n[s])); a warp reading one slice
//                                  reads contiguous 8-byte words of one component row.
//   rho_k [S][M][K]      double2  per-slice charge density sum_p exp(i k . r_pb) of each species
//                                  (species_class.h:23), only kept where a long-range action or a
//                                  structure-factor observable needs it.
//   kidx  [K]            int32    packed lattice indices (n_x, n_y, n_z) of the stored half-space
//                                  k-vectors, 8 bits each with an offset of 128.
//
// The reference's per-bead charge densities (bead_class.h:20-21, N*M*K complex numbers: 481 MB
// for the 66-electron gas and 426 GB for the 1024-electron one) are not stored: the density of a
// bead is recomputed from its position when it is needed, with the same per-dimension phase
// recurrence (k_space_class.h:83-94).
#pragma once

#include <cstdint>

namespace pimc {

constexpr int kMaxSpecies = 4;
constexpr int kMaxKinetic = 4;
constexpr int kMaxTrap = 4;
constexpr int kMaxPair = 8;
constexpr int kMaxMoves = 8;
constexpr int kMaxLevels = 12;   // bisection levels / kinetic spline levels (skip = 2^l)
constexpr int kMaxSegment = 1 << kMaxLevels;

// Phases of one bisection attempt timed by the sweep kernel's optional tracing: segment and random
// numbers, sampling chain, per-level terms, grid work, grid barrier, final sum, decision, commit.
constexpr int kSweepPhases = 8;
// Extra tracing slots: the slowest warp of each role inside phases 2-4 (cycles from the phase
// start): sampling chain, stored-copy level sums, old phase tables, stored-copy pair links,
// working-copy level sums, new phase tables, old Ewald phases, grid-phase pair links + Ewald cells.
constexpr int kSweepRoles = 8;
constexpr int kSweepTimingSlots = kSweepPhases + kSweepRoles;

// Error word values written by kernels (read back by the host as PIMC_ERR_*).
constexpr int kDevErrTimeout = 1;
constexpr int kDevErrNonFinite = 2;

/// Natural cubic interpolating spline stored as one cubic polynomial per interval:
/// f(x) = c0 + t (c1 + t (c2 + t c3)), t = x - x_i, on [x_i, x_{i+1}]; arguments are clamped to
/// [x_0, x_{n-1}]. Uniform grids locate the interval arithmetically, general grids through a
/// bucket table followed by a short forward scan.
struct alignas(32) Cubic4 {
    double c0, c1, c2, c3;
};

struct CubicTable {
    const double* x = nullptr;       // knots [n]
    const Cubic4* c = nullptr;       // interval polynomials [n-1]
    const int32_t* bucket = nullptr; // general grid: first interval of each bucket [n_bucket]
    int32_t n = 0;
    int32_t n_bucket = 0;
    int32_t uniform = 0;
    double x0 = 0., x1 = 0.;
    double inv_dx = 0.;              // uniform: 1/spacing; general: buckets per unit length
};

/// Knots of one axis of a 2-D table: uniform grids locate the cell arithmetically, general grids
/// through a bucket table followed by a short forward scan (as CubicTable).
struct GridDev {
    const double* x = nullptr;
    const int32_t* bucket = nullptr;
    int32_t n = 0, n_bucket = 0, uniform = 0;
    double x0 = 0., x1 = 0., inv_dx = 0.;
};

/// Natural bicubic interpolating spline on a rectilinear grid: the tensor product of natural cubic
/// splines, which is what einspline's NUBspline_2d_d with {NATURAL, NATURAL} conditions represents
/// (ilkka_pair_action_class.h:264-280). Stored as one bicubic polynomial per cell,
/// f = sum_{a,b} c[16 cell + 4a + b] u^a v^b with u = x - x_i, v = y - y_j, cell = i (n_y - 1) + j.
/// Outside the grid the edge cell's polynomial continues (the arguments are not clamped).
struct BicubicTable {
    GridDev gx, gy;
    const double* c = nullptr;
};

/// Components of a multi-spline on one grid (einspline's multi_NUBspline_1d_d): component m on
/// interval i is c[i n_comp + m], a natural cubic spline as CubicTable.
struct MultiCubic {
    GridDev g;
    const Cubic4* c = nullptr;
    int32_t n_comp = 0;
};

/// Kinetic action of one species (src/actions/single_action/kinetic_class.h:10-169).
struct KineticDev {
    uint32_t species = 0;
    int32_t has_images = 0;          // n_images > 0: the periodic-image splines are non-zero
    double i4lt = 0.;                // 1/(4 lambda tau)
    double i4ltt = 0.;               // 1/(4 lambda tau^2)
    double i4lt_level[kMaxLevels];   // 1/(4 lambda (tau 2^l)), the constant of spline 2^l - 1
    double d_action_d_beta_const = 0.;
    CubicTable image[kMaxLevels];    // image action of the free propagator at tau * 2^l
    CubicTable d_image_d_tau;        // its tau derivative at tau
};

/// Harmonic trap (src/actions/single_action/trap_class.h:7-65).
struct TrapDev {
    uint32_t species = 0;
    uint32_t max_level = 0;
    double cofactor_a = 0., cofactor_b = 0.;
};

constexpr int32_t kPairBare = 0;   // BarePairAction (bare_pair_action_class.h:7-183)
constexpr int32_t kPairIlkka = 1;  // IlkkaPairAction (ilkka_pair_action_class.h:7-433)
constexpr int32_t kPairDavid = 2;  // DavidPairAction (david_pair_action_class.h:7-361)

/// Pair action: the primitive BarePairAction; IlkkaPairAction's off-diagonal action u(x, y) of
/// x = q + s/2, y = q - s/2 (q = (|r| + |r'|)/2, s = |r - r'|) with its tau derivative; or
/// DavidPairAction's expansion (u_00(r) + u_00(r'))/2 + sum_kj u_kj(q) z^2j s^2(k-j), z = r - r'.
/// The bare and Ilkka actions keep the potential tables v (Potential; and DActionDBeta of the bare
/// action); the David action's potential is component 0 of its multi-splines.
struct PairDev {
    uint32_t sa = 0, sb = 0;
    int32_t kind = kPairBare;
    int32_t is_coulomb = 0, use_long_range = 0, is_constant = 0;
    uint32_t max_level = 0;
    double r_v_min = 0., r_v_max = 0., r_vl_min = 0., r_vl_max = 0.;
    double v_long_k_0 = 0., v_long_r_0 = 0.;   // already scaled as in the reference constructor
    CubicTable v_r, v_long_r;
    const double* v_long_k = nullptr;          // [K]
    // IlkkaPairAction only
    BicubicTable u_xy, du_xy;
    CubicTable u_long_r, du_long_r;
    double r_u_min = 0., r_u_max = 0., r_du_min = 0., r_du_max = 0.;
    double du_long_k_0 = 0., du_long_r_0 = 0.; // scaled as v_long_k_0 / v_long_r_0
    const double* u_long_k = nullptr;          // [K] (also DavidPairAction)
    const double* du_long_k = nullptr;         // [K] (also DavidPairAction)
    // DavidPairAction only
    MultiCubic u_kj, du_kj;                    // (max_level + 1) x (n_val + 1) components: the table of
                                               // level l from component l * kj_stride, its component 0
                                               // the potential
    uint32_t n_order = 0, kj_stride = 0;       // kj_stride = n_val + 1
    double r_d_min = 0., r_d_max = 0.;         // the grid's ends (GetLimits)
};

/// Bisection move (src/events/moves/single_species_move/bisect/bisect_class.h:8-214) with the
/// subset of actions that touch its species (move_class.h:27-31).
struct MoveDev {
    uint32_t species = 0;
    uint32_t n_level = 0;
    int32_t has_images = 0;
    double lambda = 0.;
    double i4lt_sample[kMaxLevels];            // 1/(4 lambda * tau 2^l / 2)
    CubicTable sample_image[kMaxLevels];       // image action of the sampling propagator
    int32_t n_kinetic = 0, n_trap = 0, n_pair = 0;
    int32_t kinetic[kMaxKinetic];
    int32_t trap[kMaxTrap];
    int32_t pair[kMaxPair];
};

struct SystemDev {
    uint32_t n_d = 3, M = 0, S = 0, n_total = 0, n_pad = 0;
    int32_t pbc = 1;
    double L = 0., iL = 0., tau = 0., beta = 0., vol = 1.;
    uint32_t sp_off[kMaxSpecies] = {0};
    uint32_t sp_n[kMaxSpecies] = {0};
    double sp_lambda[kMaxSpecies] = {0};
    int32_t sp_rho[kMaxSpecies] = {0};         // rho_k slot of each species, -1 when not kept

    double* pos = nullptr;      // committed ("old") copy  [M][3][n_pad]
    double* pos_new = nullptr;  // proposal ("new") copy   [M][3][n_pad]
    // Path permutation at the ring closure: bead (g, M - 1) is followed by bead (perm[g], 0)
    // (bead_class.h:38-41 links after the relabelling of perm_bisect_class.h:47-56); perm_inv is
    // its inverse. Identity without exchanges.
    const uint32_t* perm = nullptr;      // [n_total]
    const uint32_t* perm_inv = nullptr;  // [n_total]

    uint32_t K = 0;
    int32_t max_index[3] = {0, 0, 0};
    double box[3] = {0., 0., 0.};
    const int32_t* kidx = nullptr;   // [K]
    double2* rho_k = nullptr;        // [n_rho][M][K]

    int32_t n_kinetic = 0, n_trap = 0, n_pair = 0;
    KineticDev kinetic[kMaxKinetic];
    TrapDev trap[kMaxTrap];
    PairDev pair[kMaxPair];
};

__host__ __device__ inline int32_t PackK(int nx, int ny, int nz) {
    return (int32_t)((uint32_t)(nx + 128) | ((uint32_t)(ny + 128) << 8) | ((uint32_t)(nz + 128) << 16));
}

}  // namespace pimc
