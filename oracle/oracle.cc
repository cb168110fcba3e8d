// ORACLE — test infrastructure only. Nothing in the product library links, loads or calls this file;
// it is the CPU checker used by tests/, the smoke check and the bench's CPU-baseline leg.
//
// A plain C++/FP64 restatement of simpimc's action/move/estimator hot path, written to follow the
// reference's own loops and quirks one for one. Each class cites the reference file:line it restates.
// The reference itself cannot be built here: it needs the scaffold submodule (empty), Armadillo,
// HDF5, einspline (fetched from an unpinned master tarball) and MPI. Its repository holds no unit
// tests, fixtures or golden vectors for this path. Parity is therefore pinned through known answers
// instead: the exact discrete-path energy of harmonic oscillators (the reference's inputs/sho case
// and the trapped-particle configuration), Philox known-answer vectors, natural-spline identities
// and independent Ewald sums (tests/test_oracle_*.py).
//
// Deliberate departures from the reference:
//  * einspline's natural-BC cubic B-splines are represented as the (identical) natural cubic
//    interpolating splines; 1-D table arguments are clamped to the grid, and the 2-D table of
//    IlkkaPairAction continues its edge cells outside it.
//  * The scaffold RNG is replaced by the Philox draw protocol shared with the GPU path.
//  * k-vectors are enumerated lexicographically (the reference's GenCombPermK order is unavailable);
//    only the summation order differs.
//  * Open boundaries (pbc=0) skip k-space setup (the reference divides by L=0 there).
//  * Permutations are not modelled: beads link to the same particle on neighbouring slices.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../simpimc_gb300/src/framework/input.h"
#include "../simpimc_gb300/src/framework/table_io.h"

namespace orc {

using pimc::Input;
using pimc::InputError;
using pimc::TableFile;
typedef std::complex<double> cplx;

// ---------------------------------------------------------------------------------------------
// Philox4x32-10, written out independently of the product's copy (same published algorithm).
struct RNG4 {
    uint32_t w[4];
};

static RNG4 philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
    uint32_t x0 = c[0], x1 = c[1], x2 = c[2], x3 = c[3];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * x0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * x2;
        uint32_t y0 = (uint32_t)(p1 >> 32) ^ x1 ^ k0;
        uint32_t y1 = (uint32_t)p1;
        uint32_t y2 = (uint32_t)(p0 >> 32) ^ x3 ^ k1;
        uint32_t y3 = (uint32_t)p0;
        x0 = y0;
        x1 = y1;
        x2 = y2;
        x3 = y3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    RNG4 o = {{x0, x1, x2, x3}};
    return o;
}

struct Stream {
    uint32_t seed, chain, move;
    uint64_t attempt;
    RNG4 block(uint32_t b) const {
        uint32_t c[4] = {(uint32_t)attempt, (uint32_t)(attempt >> 32), move, b};
        return philox(c, seed, chain);
    }
};

static uint32_t uidx(uint32_t w, uint32_t n) { return (uint32_t)(((uint64_t)w * n) >> 32); }

// The move's exactly specified binary32 transforms (this file is compiled with
// -ffp-contract=off; every fused multiply-add is an explicit fmaf): a 24-bit uniform, the
// logarithm by m in [sqrt(1/2), sqrt(2)) and 2 atanh((m-1)/(m+1)), sin/cos of 2 pi u by quadrant
// reduction and Taylor polynomials, Box-Muller normals.
static float u24(uint32_t w) { return (float)(w >> 8) * (1.0f / 16777216.0f); }

static float logf_spec(float x) {
    if (x == 0.f) return -INFINITY;
    uint32_t b;
    std::memcpy(&b, &x, 4);
    int e = (int)((b >> 23) & 0xffu) - 126;
    uint32_t mb = (b & 0x007fffffu) | 0x3f000000u;
    float m;
    std::memcpy(&m, &mb, 4);
    if (m < 0.70710678f) {
        m = m + m;
        e -= 1;
    }
    const float f = m - 1.0f;
    const float s = f / (2.0f + f);
    const float s2 = s * s;
    float p = std::fmaf(s2, 1.0f / 9.0f, 1.0f / 7.0f);
    p = std::fmaf(s2, p, 1.0f / 5.0f);
    p = std::fmaf(s2, p, 1.0f / 3.0f);
    p = s2 * p;
    const float two_s = s + s;
    const float lm = std::fmaf(two_s, p, two_s);
    const float ef = (float)e;
    return std::fmaf(ef, 0.693145751953125f, std::fmaf(ef, 1.428606765330187e-06f, lm));
}

static void sincos2pi_spec(float u, float& s, float& c) {
    const float v = u * 4.0f;
    const float q = std::floor(v);
    const float f = v - q;
    const int qi = (int)q & 3;
    const float t = (f - 0.5f) * 1.57079637f;
    const float t2 = t * t;
    float ps = std::fmaf(t2, 1.0f / 362880.0f, -1.0f / 5040.0f);
    ps = std::fmaf(t2, ps, 1.0f / 120.0f);
    ps = std::fmaf(t2, ps, -1.0f / 6.0f);
    ps = t2 * ps;
    const float st = std::fmaf(t, ps, t);
    float pc = std::fmaf(t2, -1.0f / 3628800.0f, 1.0f / 40320.0f);
    pc = std::fmaf(t2, pc, -1.0f / 720.0f);
    pc = std::fmaf(t2, pc, 1.0f / 24.0f);
    pc = std::fmaf(t2, pc, -0.5f);
    const float ct = std::fmaf(t2, pc, 1.0f);
    const float sp = (st + ct) * 0.70710678f;
    const float cp = (ct - st) * 0.70710678f;
    switch (qi) {
        case 0: s = sp; c = cp; break;
        case 1: s = cp; c = -sp; break;
        case 2: s = -sp; c = -cp; break;
        default: s = -cp; c = sp; break;
    }
}

static void boxmuller(uint32_t w0, uint32_t w1, float& z0, float& z1) {
    const float u0 = u24(w0), u1 = u24(w1);
    const float r = std::sqrt(-2.0f * logf_spec(1.0f - u0));
    float s, c;
    sincos2pi_spec(u1, s, c);
    z0 = r * c;
    z1 = r * s;
}

// ---------------------------------------------------------------------------------------------
// Natural cubic interpolating spline (stands in for einspline UBspline_1d_d / NUBspline_1d_d with
// {NATURAL, NATURAL} boundary conditions: free_spline_class.h:64-67, bare_pair_action_class.h:36-67).
struct Spline {
    std::vector<double> x, y, m;  // knots, values, second derivatives
    bool uniform = false;
    double x0 = 0., dx = 1.;

    void Build(const std::vector<double>& xs, const std::vector<double>& ys, bool is_uniform) {
        x = xs;
        y = ys;
        uniform = is_uniform;
        size_t n = x.size();
        m.assign(n, 0.);
        if (uniform) {
            x0 = x[0];
            dx = (x[n - 1] - x[0]) / (double)(n - 1);
        }
        if (n < 3) return;
        std::vector<double> c(n, 0.), d(n, 0.);
        // Thomas algorithm on rows 1..n-2 with m_0 = m_{n-1} = 0.
        for (size_t i = 1; i + 1 < n; ++i) {
            double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
            double a = h0, b = 2. * (h0 + h1), cc = h1;
            double r = 6. * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
            if (i > 1) {
                b -= a * c[i - 1];
                r -= a * d[i - 1];
            }
            c[i] = cc / b;
            d[i] = r / b;
        }
        m[n - 2] = d[n - 2];
        for (size_t i = n - 2; i-- > 1;) m[i] = d[i] - c[i] * m[i + 1];
    }

    size_t Interval(double& t) const {
        size_t n = x.size();
        if (t < x[0]) t = x[0];
        if (t > x[n - 1]) t = x[n - 1];
        size_t i;
        if (uniform) {
            double f = std::floor((t - x0) / dx);
            i = f < 0. ? 0 : (size_t)f;
            if (i > n - 2) i = n - 2;
        } else {
            i = (size_t)(std::upper_bound(x.begin(), x.end(), t) - x.begin());
            i = i == 0 ? 0 : i - 1;
            if (i > n - 2) i = n - 2;
        }
        return i;
    }

    double Eval(double t) const {
        size_t i = Interval(t);
        double h = x[i + 1] - x[i];
        double A = (x[i + 1] - t) / h, B = 1. - A;
        return A * y[i] + B * y[i + 1] + ((A * A * A - A) * m[i] + (B * B * B - B) * m[i + 1]) * h * h / 6.;
    }

    void EvalVG(double t, double& v, double& g) const {
        size_t i = Interval(t);
        double h = x[i + 1] - x[i];
        double A = (x[i + 1] - t) / h, B = 1. - A;
        v = A * y[i] + B * y[i + 1] + ((A * A * A - A) * m[i] + (B * B * B - B) * m[i + 1]) * h * h / 6.;
        g = (y[i + 1] - y[i]) / h + (-(3. * A * A - 1.) * m[i] + (3. * B * B - 1.) * m[i + 1]) * h / 6.;
    }

    // Value and slope without clamping the argument: outside the knots the edge interval's cubic
    // continues.
    void EvalExtVG(double t, double& v, double& g) const {
        size_t n = x.size();
        size_t i = (size_t)(std::upper_bound(x.begin(), x.end(), t) - x.begin());
        i = i == 0 ? 0 : i - 1;
        if (i > n - 2) i = n - 2;
        double h = x[i + 1] - x[i];
        double A = (x[i + 1] - t) / h, B = 1. - A;
        v = A * y[i] + B * y[i + 1] + ((A * A * A - A) * m[i] + (B * B * B - B) * m[i + 1]) * h * h / 6.;
        g = (y[i + 1] - y[i]) / h + (-(3. * A * A - 1.) * m[i] + (3. * B * B - 1.) * m[i + 1]) * h / 6.;
    }
};

// 2-D natural spline on a rectilinear grid: the tensor product of natural cubic splines that
// einspline's NUBspline_2d_d with {NATURAL, NATURAL} conditions represents. It is evaluated by its
// definition as a product of 1-D interpolations: a natural spline along x within every grid row
// y_j, then a natural spline along y through those row values (and through their x slopes for
// df/dx). Outside the grid each 1-D spline continues its edge interval's cubic.
struct Spline2 {
    std::vector<double> y;
    std::vector<Spline> rows;  // rows[j]: the spline in x of f(., y_j)

    void Build(const std::vector<double>& xs, const std::vector<double>& ys, const std::vector<double>& f) {
        size_t nx = xs.size(), ny = ys.size();
        if (nx < 2 || ny < 2 || f.size() != nx * ny) throw InputError("2-D spline: inconsistent grid and values");
        y = ys;
        rows.assign(ny, Spline());
        std::vector<double> col(nx);
        for (size_t j = 0; j < ny; ++j) {
            for (size_t i = 0; i < nx; ++i) col[i] = f[i * ny + j];  // value (i, j) at i n_y + j
            rows[j].Build(xs, col, false);
        }
    }

    void EvalVG(double xx, double yy, double& f, double& fx, double& fy) const {
        size_t ny = y.size();
        std::vector<double> v(ny), dv(ny);
        for (size_t j = 0; j < ny; ++j) rows[j].EvalExtVG(xx, v[j], dv[j]);
        Spline sv, sd;
        sv.Build(y, v, false);
        sd.Build(y, dv, false);
        double unused;
        sv.EvalExtVG(yy, f, fy);
        sd.EvalExtVG(yy, fx, unused);
    }

    double Eval(double xx, double yy) const {
        double f, fx, fy;
        EvalVG(xx, yy, f, fx, fy);
        return f;
    }
};

// ---------------------------------------------------------------------------------------------
// KSpace (src/data_structures/k_space_class.h:5-95).
struct KSpace {
    double cutoff = 0.;
    double L = 0.;
    uint32_t n_d = 3;
    std::vector<double> mags;
    std::vector<std::vector<double>> vecs;
    std::vector<std::vector<int>> indices;
    std::vector<double> box;
    std::vector<int> max_index;
    std::vector<std::vector<cplx>> c_k;

    // k_space_class.h:17-30 — half-space selection.
    bool Include(const std::vector<double>& k, double k_cut) const {
        double k2 = 0.;
        for (double x : k) k2 += x * x;
        if (k2 < k_cut * k_cut && k2 != 0.) {
            if (k[0] > 0.) return true;
            if (n_d >= 2 && (k[0] == 0. && k[1] > 0.)) return true;
            if (n_d >= 3 && (k[0] == 0. && k[1] == 0. && k[2] > 0.)) return true;
            return false;
        }
        return false;
    }

    // k_space_class.h:33-80. Enumeration order is lexicographic in (n_0, n_1, n_2).
    void Setup(double k_cut) {
        if (L == 0.) return;  // open boundaries: no k-space
        if (k_cut <= cutoff) return;
        vecs.clear();
        indices.clear();
        mags.clear();
        cutoff = k_cut;
        box.assign(n_d, 2. * M_PI / L);
        max_index.assign(n_d, 0);
        for (uint32_t d = 0; d < n_d; ++d) max_index[d] = (int)(uint32_t)std::ceil(1.1 * k_cut / box[d]);
        c_k.assign(n_d, {});
        for (uint32_t d = 0; d < n_d; ++d) c_k[d].assign(2 * max_index[d] + 1, cplx(0., 0.));
        std::vector<int> n(n_d, 0);
        std::vector<int> lo(n_d), hi(n_d);
        for (uint32_t d = 0; d < n_d; ++d) {
            lo[d] = -max_index[d];
            hi[d] = max_index[d];
        }
        for (uint32_t d = 0; d < n_d; ++d) n[d] = lo[d];
        for (;;) {
            std::vector<double> k(n_d);
            std::vector<int> ki(n_d);
            for (uint32_t d = 0; d < n_d; ++d) {
                k[d] = n[d] * box[d];
                ki[d] = max_index[d] + n[d];
            }
            if (Include(k, k_cut)) {
                double k2 = 0.;
                for (double x : k) k2 += x * x;
                vecs.push_back(k);
                indices.push_back(ki);
                mags.push_back(std::sqrt(k2));
            }
            int d = (int)n_d - 1;
            while (d >= 0) {
                if (++n[d] <= hi[d]) break;
                n[d] = lo[d];
                --d;
            }
            if (d < 0) break;
        }
    }

    // k_space_class.h:83-94.
    void CalcC(const double* r) { CalcCInto(r, c_k); }
    void CalcCInto(const double* r, std::vector<std::vector<cplx>>& ck) const {
        for (uint32_t d = 0; d < box.size(); ++d) {
            double phi = r[d] * box[d];
            cplx t(std::cos(phi), std::sin(phi));
            int m = max_index[d];
            ck[d][m] = 1.;
            for (int k = 1; k <= m; ++k) {
                ck[d][m + k] = t * ck[d][m + k - 1];
                ck[d][m - k] = std::conj(ck[d][m + k]);
            }
        }
    }

    size_t K() const { return vecs.size(); }
};

enum Mode { OLD_MODE = 0, NEW_MODE = 1 };

struct Path;

// ---------------------------------------------------------------------------------------------
// Species (src/data_structures/species_class.h:7-446) with the bead grid of bead_class.h.
struct Species {
    std::string name;
    uint32_t s_i = 0, n_part = 0, n_bead = 0, n_d = 3, offset = 0;
    double lambda = 0.;
    bool fermi = false, fixed_node = false;
    bool need_update_rho_k = true;
    // Per-slice charge densities and their copies (species_class.h:23-24): [b][k].
    std::vector<cplx> rho_k, rho_k_c;
    // Per-bead charge densities and their copies (bead_class.h:20-21): [p][b][k].
    std::vector<cplx> bead_rho_k, bead_rho_k_c;
    // Bead links (bead_class.h:38-41, 98-111): bead (p, b) is followed by bead (nxt[p M + b], b + 1 mod M);
    // OLD mode reads the copy nxt_c. Between moves every link keeps its particle label except at the
    // ring closure b = M - 1, which holds the path permutation (AssignParticleLabels,
    // perm_bisect_class.h:47-56, relabels the beads after an accepted permutation).
    std::vector<uint32_t> nxt, nxt_c;
    uint32_t bead_loop(uint32_t b) const { return b >= n_bead ? b - n_bead : b; }  // species_class.h:101
};

// Lean densities (no reference counterpart; a memory option of this oracle): the reference keeps every
// bead's density and its copy (bead_class.h:20-21), N M K complex numbers twice, which is 426 GB for
// N = 1024, M = 512, K = 25398. With lean densities on, a Path keeps only the per-slice densities
// and recomputes a bead's density from its position wherever the reference reads the stored one.
// The stored density always equals CalcRhoK of the bead's position of that copy, so the results are
// identical bit for bit. The per-slice sums at initialisation run over slices in parallel (OpenMP),
// each slice summing its particles in order as the reference does. Set before oracle_create.
static bool g_lean_densities = false;

struct Path {
    uint32_t n_d = 3, n_bead = 0;
    bool lean_rho = g_lean_densities;
    double beta = 0., L = 0., iL = 0., vol = 1., tau = 0.;
    bool pbc = true;
    Mode mode = NEW_MODE;
    KSpace ks;
    std::vector<Species> species;
    uint32_t n_total = 0;
    std::vector<double> r, r_c;  // positions (new) and copies (old): [n_total][n_bead][n_d]

    Path(const Input& in) {
        // path_class.h:25-62
        Input sys = in.GetChild("System");
        n_d = sys.GetAttribute<uint32_t>("n_d");
        n_bead = sys.GetAttribute<uint32_t>("n_bead");
        beta = sys.GetAttribute<double>("beta");
        pbc = sys.GetAttribute<bool>("pbc", true);
        L = sys.GetAttribute<double>("L", 0.);
        if (n_d < 1 || n_d > 3) throw InputError("n_d must be 1, 2 or 3");
        if (n_bead < 2) throw InputError("n_bead must be at least 2");
        if (pbc) {
            if (!(L > 0.)) throw InputError("pbc=1 needs a positive L");
            iL = 1. / L;
            vol = std::pow(L, n_d);
        } else {
            L = 0.;
            iL = 0.;
            vol = 1.;
        }
        tau = beta / (1. * n_bead);
        ks.n_d = n_d;
        ks.L = L;
        ks.cutoff = 0.;
        if (pbc) ks.Setup(sys.GetAttribute<double>("k_cut", 2. * M_PI / L));
        for (auto& sin : in.GetChild("Particles").GetChildList("Species")) {
            Species s;
            s.name = sin.GetAttribute<std::string>("name");
            s.n_part = sin.GetAttribute<uint32_t>("n_part");
            s.lambda = sin.GetAttribute<double>("lambda");
            s.fermi = sin.GetAttribute<bool>("fermi", false);
            s.fixed_node = sin.GetAttribute<bool>("fixed_node", false);
            s.s_i = (uint32_t)species.size();
            s.n_bead = n_bead;
            s.n_d = n_d;
            s.offset = n_total;
            n_total += s.n_part;
            species.push_back(s);
        }
        r.assign((size_t)n_total * n_bead * n_d, 0.);
        r_c = r;
        for (auto& s : species) {
            s.nxt.resize((size_t)s.n_part * n_bead);
            for (uint32_t p = 0; p < s.n_part; ++p)
                for (uint32_t b = 0; b < n_bead; ++b) s.nxt[(size_t)p * n_bead + b] = p;
            s.nxt_c = s.nxt;
        }
    }

    Species& GetSpecies(const std::string& nm) {
        for (auto& s : species)
            if (s.name == nm) return s;
        throw InputError("no species named '" + nm + "'");
    }

    size_t Idx(const Species& s, uint32_t p, uint32_t b) const { return (((size_t)(s.offset + p)) * n_bead + s.bead_loop(b)) * n_d; }
    double* GetR(const Species& s, uint32_t p, uint32_t b) { return (mode == NEW_MODE ? r.data() : r_c.data()) + Idx(s, p, b); }
    double* GetRMode(const Species& s, uint32_t p, uint32_t b, Mode m) { return (m == NEW_MODE ? r.data() : r_c.data()) + Idx(s, p, b); }

    // Label of the bead after (p, b) (GetNextBead(1), bead_class.h:22-23, 104).
    uint32_t NextLabel(const Species& s, uint32_t p, uint32_t b, Mode m) const {
        return (m == NEW_MODE ? s.nxt : s.nxt_c)[(size_t)p * n_bead + s.bead_loop(b)];
    }
    // Label of the bead before (p, b) (GetPrevBead(1)): the bead whose link reaches (p, b).
    uint32_t PrevLabel(const Species& s, uint32_t p, uint32_t b, Mode m) const {
        const uint32_t bp = (s.bead_loop(b) + n_bead - 1) % n_bead;
        for (uint32_t q = 0; q < s.n_part; ++q)
            if (NextLabel(s, q, bp, m) == p) return q;
        throw std::logic_error("bead links are not a permutation");
    }
    // GetNextBead(n) / GetPrevBead(n) of bead (p, b): returns the label and sets `slice`.
    uint32_t Walk(const Species& s, uint32_t p, uint32_t b, uint32_t n, Mode m, uint32_t& slice) const {
        uint32_t q = p, bb = s.bead_loop(b);
        for (uint32_t i = 0; i < n; ++i) {
            q = NextLabel(s, q, bb, m);
            bb = bb + 1 == n_bead ? 0 : bb + 1;
        }
        slice = bb;
        return q;
    }
    uint32_t WalkBack(const Species& s, uint32_t p, uint32_t b, uint32_t n, Mode m, uint32_t& slice) const {
        uint32_t q = p, bb = s.bead_loop(b);
        for (uint32_t i = 0; i < n; ++i) {
            q = PrevLabel(s, q, bb, m);
            bb = bb == 0 ? n_bead - 1 : bb - 1;
        }
        slice = bb;
        return q;
    }
    // The path permutation of a species: pi[p] = label of the bead after (p, M - 1).
    std::vector<uint32_t> Closure(const Species& s) const {
        std::vector<uint32_t> pi(s.n_part);
        for (uint32_t p = 0; p < s.n_part; ++p) pi[p] = NextLabel(s, p, n_bead - 1, NEW_MODE);
        return pi;
    }
    // Species::GetSign (species_class.h:149-157) over every species (path_class.h:169-175).
    int GetSign() const {
        int sign = 1;
        for (const auto& s : species) {
            if (!s.fermi) continue;
            std::vector<char> seen(s.n_part, 0);
            for (uint32_t p = 0; p < s.n_part; ++p) {
                if (seen[p]) continue;
                uint32_t len = 0, q = p;
                do {
                    seen[q] = 1;
                    q = NextLabel(s, q, n_bead - 1, NEW_MODE);
                    ++len;
                } while (q != p);
                if (!(len % 2)) sign = -sign;
            }
        }
        return sign;
    }

    // path_class.h:131-134
    void PutInBox(double* x) const {
        for (uint32_t d = 0; d < n_d; ++d) x[d] -= std::nearbyint(x[d] * iL) * L;
    }
    // path_class.h:108-112
    void Dr(const double* r0, const double* r1, double* dr) const {
        for (uint32_t d = 0; d < n_d; ++d) dr[d] = r0[d] - r1[d];
        PutInBox(dr);
    }
    // path_class.h:137-150
    void DrDrpDrrp(uint32_t b0, uint32_t b1, const Species& s0, const Species& s1, uint32_t p0, uint32_t p1, double& r_mag,
                   double& r_p_mag, double& r_r_p_mag) {
        double rv[3], rp[3], rrp[3];
        const double* a0 = GetR(s1, p1, b0);
        const double* c0 = GetR(s0, p0, b0);
        const double* a1 = GetR(s1, p1, b1);
        const double* c1 = GetR(s0, p0, b1);
        for (uint32_t d = 0; d < n_d; ++d) {
            rv[d] = a0[d] - c0[d];
            rp[d] = a1[d] - c1[d];
        }
        for (uint32_t d = 0; d < n_d; ++d) {
            rv[d] -= std::nearbyint(rv[d] * iL) * L;
            rp[d] += std::nearbyint((rv[d] - rp[d]) * iL) * L;
        }
        for (uint32_t d = 0; d < n_d; ++d) rrp[d] = rv[d] - rp[d];
        for (uint32_t d = 0; d < n_d; ++d) rrp[d] -= std::nearbyint(rrp[d] * iL) * L;
        double a = 0., b = 0., c = 0.;
        for (uint32_t d = 0; d < n_d; ++d) {
            a += rv[d] * rv[d];
            b += rp[d] * rp[d];
            c += rrp[d] * rrp[d];
        }
        r_mag = std::sqrt(a);
        r_p_mag = std::sqrt(b);
        r_r_p_mag = std::sqrt(c);
    }

    // bead_class.h:125-133 — rho_k of one bead from the current-mode position.
    void CalcBeadRhoK(Species& s, uint32_t p, uint32_t b, cplx* out) {
        ks.CalcC(GetR(s, p, b));
        for (size_t k = 0; k < ks.K(); ++k) {
            cplx f = 1.;
            for (uint32_t d = 0; d < ks.n_d; ++d) f *= ks.c_k[d][ks.indices[k][d]];
            out[k] = f;
        }
    }

    // Density of bead (p, b) of copy m from its position, into `out` with the caller's phase tables.
    void BeadRhoKAt(Species& s, uint32_t p, uint32_t b, Mode m, cplx* out, std::vector<std::vector<cplx>>& ck) const {
        const double* rr = (m == NEW_MODE ? r.data() : r_c.data()) + ((size_t)(s.offset + p) * n_bead + s.bead_loop(b)) * n_d;
        ks.CalcCInto(rr, ck);
        for (size_t k = 0; k < ks.K(); ++k) {
            cplx f = 1.;
            for (uint32_t d = 0; d < ks.n_d; ++d) f *= ck[d][ks.indices[k][d]];
            out[k] = f;
        }
    }

    // The stored density of bead (p, b) of copy m; with lean densities, recomputed into `tmp`.
    cplx* BeadRhoK(Species& s, uint32_t p, uint32_t b, Mode m, std::vector<cplx>* tmp = nullptr) {
        size_t K = ks.K();
        if (lean_rho) {
            if (!tmp) throw std::logic_error("lean densities need a buffer");
            tmp->resize(K);
            std::vector<std::vector<cplx>> ck = ks.c_k;
            BeadRhoKAt(s, p, b, m, tmp->data(), ck);
            return tmp->data();
        }
        size_t off = ((size_t)p * n_bead + s.bead_loop(b)) * K;
        return (m == NEW_MODE ? s.bead_rho_k.data() : s.bead_rho_k_c.data()) + off;
    }

    // species_class.h:380-403
    void InitRhoK(Species& s) {
        size_t K = ks.K();
        s.rho_k.assign((size_t)n_bead * K, cplx(0., 0.));
        if (lean_rho && K) {
            std::vector<cplx>().swap(s.bead_rho_k);
            std::vector<cplx>().swap(s.bead_rho_k_c);
#pragma omp parallel
            {
                std::vector<std::vector<cplx>> ck = ks.c_k;
                std::vector<cplx> br(K);
#pragma omp for schedule(dynamic, 1)
                for (int64_t b = 0; b < (int64_t)n_bead; ++b) {
                    cplx* sr = &s.rho_k[(size_t)b * K];
                    for (uint32_t p = 0; p < s.n_part; ++p) {
                        BeadRhoKAt(s, p, (uint32_t)b, NEW_MODE, br.data(), ck);
                        for (size_t k = 0; k < K; ++k) sr[k] += br[k];
                    }
                }
            }
            s.rho_k_c = s.rho_k;
            return;
        }
        s.bead_rho_k.assign((size_t)s.n_part * n_bead * K, cplx(0., 0.));
        if (K == 0) {
            s.rho_k_c = s.rho_k;
            s.bead_rho_k_c = s.bead_rho_k;
            return;
        }
        Mode keep = mode;
        mode = NEW_MODE;
        for (uint32_t b = 0; b < n_bead; ++b)
            for (uint32_t p = 0; p < s.n_part; ++p) CalcBeadRhoK(s, p, b, BeadRhoK(s, p, b, NEW_MODE));
        for (uint32_t b = 0; b < n_bead; ++b)
            for (uint32_t p = 0; p < s.n_part; ++p) {
                const cplx* br = BeadRhoK(s, p, b, NEW_MODE);
                cplx* sr = &s.rho_k[(size_t)b * K];
                for (size_t k = 0; k < K; ++k) sr[k] += br[k];
            }
        s.rho_k_c = s.rho_k;
        s.bead_rho_k_c = s.bead_rho_k;
        mode = keep;
    }

    // species_class.h:406-425 (NEW mode only)
    void UpdateRhoK(Species& s, uint32_t b0, uint32_t b1, const std::vector<uint32_t>& parts, uint32_t level) {
        size_t K = ks.K();
        uint32_t skip = 1u << level;
        for (uint32_t b = b0; b < b1; b += skip) {
            uint32_t bb = s.bead_loop(b);
            std::copy(s.rho_k_c.begin() + (size_t)bb * K, s.rho_k_c.begin() + (size_t)(bb + 1) * K, s.rho_k.begin() + (size_t)bb * K);
        }
        std::vector<cplx> tn, to;
        for (uint32_t p : parts) {
            for (uint32_t b = b0; b < b1; b += skip) {
                cplx* nw = BeadRhoK(s, p, b, NEW_MODE, &tn);
                if (!lean_rho) CalcBeadRhoK(s, p, b, nw);  // lean: already formed from the NEW position
                const cplx* od = BeadRhoK(s, p, b, OLD_MODE, &to);
                cplx* sr = &s.rho_k[(size_t)s.bead_loop(b) * K];
                for (size_t k = 0; k < K; ++k) sr[k] += nw[k] - od[k];
            }
        }
        s.need_update_rho_k = false;
    }

    const std::vector<cplx>& GetRhoK(const Species& s) const { return mode == NEW_MODE ? s.rho_k : s.rho_k_c; }
};

typedef std::vector<std::pair<uint32_t, uint32_t>> Particles;  // (species index, particle index)

static double CMag2(const cplx& a, const cplx& b) { return a.real() * b.real() + a.imag() * b.imag(); }

// ---------------------------------------------------------------------------------------------
// FreeSpline (src/actions/free_spline_class.h:25-122).
struct FreeSpline {
    double i_4_lambda_tau = 0., i_4_lambda_tau_tau = 0.;
    Spline image_action, d_image_action_d_tau;
    bool has_dtau = false;

    FreeSpline() {}
    FreeSpline(double L, uint32_t n_images, double lambda, double tau, bool use_tau_derivative) {
        i_4_lambda_tau = 1. / (4. * lambda * tau);
        i_4_lambda_tau_tau = 1. / (4. * lambda * tau * tau);
        double t_l = L == 0. ? 1000. : L;
        const uint32_t num = 10000;
        double start = -t_l / 2., end = t_l / 2.;
        double dr = (end - start) / (num - 1);
        std::vector<double> xs(num), ia(num, 0.), dia(num, 0.);
        for (uint32_t i = 0; i < num; ++i) {
            double r = start + i * dr;
            xs[i] = r;
            double r2 = r * r * i_4_lambda_tau;
            for (uint32_t image = 1; image <= n_images; ++image) {
                double rp = r + image * t_l;
                double dp = r2 - rp * rp * i_4_lambda_tau;
                double ep = std::exp(dp);
                double rm = r - image * t_l;
                double dm = r2 - rm * rm * i_4_lambda_tau;
                double em = std::exp(dm);
                ia[i] += ep + em;
                if (use_tau_derivative) dia[i] += (dp * ep + dm * em) / tau;
            }
            if (use_tau_derivative) dia[i] = dia[i] / (1. + ia[i]);
            ia[i] = -std::log1p(ia[i]);
        }
        image_action.Build(xs, ia, true);
        if (use_tau_derivative) {
            d_image_action_d_tau.Build(xs, dia, true);
            has_dtau = true;
        }
    }

    double GetLogRhoFree(const double* r, uint32_t n_d) const {
        double tot = 0., r2 = 0.;
        for (uint32_t d = 0; d < n_d; ++d) {
            tot -= image_action.Eval(r[d]);
            r2 += r[d] * r[d];
        }
        return tot - r2 * i_4_lambda_tau;
    }
    double GetDLogRhoFreeDTau(const double* r, uint32_t n_d) const {
        double tot = 0., r2 = 0.;
        for (uint32_t d = 0; d < n_d; ++d) {
            tot -= d_image_action_d_tau.Eval(r[d]);
            r2 += r[d] * r[d];
        }
        return tot - r2 * i_4_lambda_tau_tau;
    }
};

// ---------------------------------------------------------------------------------------------
// Action base (src/actions/action_class.h:7-74).
struct Action {
    Path& path;
    std::string name, type;
    int n_images = 0;
    uint32_t max_level = 0;
    bool is_importance_weight = false;
    std::vector<uint32_t> species_list;

    Action(Path& p, const Input& in) : path(p) {
        name = in.GetAttribute<std::string>("name");
        type = in.GetAttribute<std::string>("type");
        n_images = in.GetAttribute<int>("n_images", 0);
        max_level = in.GetAttribute<uint32_t>("max_level", 0);
    }
    virtual ~Action() {}
    virtual double DActionDBeta() { return 0.; }
    virtual double VirialEnergy(double) { return DActionDBeta(); }
    virtual double GetAction(uint32_t, uint32_t, const Particles&, uint32_t) { return 0.; }
    virtual void GetActionGradient(uint32_t, uint32_t, const Particles&, uint32_t, double* g) {
        for (uint32_t d = 0; d < path.n_d; ++d) g[d] = 0.;
    }
    virtual double Potential() { return 0.; }
    virtual void Accept() {}
    virtual void Reject() {}
};

// src/actions/single_action/single_action_class.h:7-24
struct SingleAction : Action {
    double i_4_lambda_tau;
    Species* species;
    SingleAction(Path& p, const Input& in) : Action(p, in) {
        species = &p.GetSpecies(in.GetAttribute<std::string>("species"));
        i_4_lambda_tau = 1. / (4. * species->lambda * p.tau);
        species_list.push_back(species->s_i);
    }
};

// src/actions/single_action/kinetic_class.h:10-169
struct Kinetic : SingleAction {
    double d_action_d_beta_const;
    std::vector<FreeSpline> rho_free_splines;

    Kinetic(Path& p, const Input& in) : SingleAction(p, in) {
        d_action_d_beta_const = species->n_part * species->n_bead * p.n_d / (2. * p.tau);
        // kinetic_class.h:16-24
        uint32_t n_spline = species->n_bead / 2 + (species->n_bead % 2) + 1;
        rho_free_splines.resize(n_spline);
        rho_free_splines[0] = FreeSpline(p.L, n_images, species->lambda, p.tau, true);
        for (uint32_t i = 1; i < n_spline; ++i) rho_free_splines[i] = FreeSpline(p.L, n_images, species->lambda, p.tau * (i + 1), false);
    }

    // kinetic_class.h:35-45
    double DActionDBeta() override {
        double tot = d_action_d_beta_const;
        double dr[3];
        for (uint32_t b = 0; b < species->n_bead; ++b)
            for (uint32_t p = 0; p < species->n_part; ++p) {
                const uint32_t q = path.NextLabel(*species, p, b, path.mode);
                path.Dr(path.GetR(*species, p, b), path.GetR(*species, q, b + 1), dr);
                tot += rho_free_splines[0].GetDLogRhoFreeDTau(dr, path.n_d);
            }
        return tot;
    }

    // kinetic_class.h:48-102 (beads b_0, b_1, b_2 follow the links)
    double VirialEnergy(double window) override {
        uint32_t n_d = path.n_d, M = species->n_bead;
        const Mode m = path.mode;
        double tot = d_action_d_beta_const / window;
        struct B {
            uint32_t p, b;
        };
        auto next = [&](B x) { return B{path.NextLabel(*species, x.p, x.b, m), (x.b + 1) % M}; };
        auto R = [&](B x) { return path.GetR(*species, x.p, x.b); };
        for (uint32_t p = 0; p < species->n_part; ++p) {
            B b0{p, 0};
            B b1 = next(b0);
            B b2 = next(b1);
            double dr1[3], drL[3], t[3];
            path.Dr(R(b1), R(b0), dr1);
            for (uint32_t d = 0; d < n_d; ++d) drL[d] = dr1[d];
            for (uint32_t s = 1; s < window; ++s) {
                path.Dr(R(b2), R(b1), t);
                for (uint32_t d = 0; d < n_d; ++d) drL[d] += t[d];
                b1 = b2;
                b2 = next(b2);
            }
            double dot = 0.;
            for (uint32_t d = 0; d < n_d; ++d) dot += drL[d] * dr1[d];
            tot -= dot * i_4_lambda_tau / (window * path.tau);
            for (uint32_t b = 1; b < M; ++b) {
                for (uint32_t d = 0; d < n_d; ++d) drL[d] -= dr1[d];
                path.Dr(R(b2), R(b1), t);
                for (uint32_t d = 0; d < n_d; ++d) drL[d] += t[d];
                b0 = next(b0);
                path.Dr(R(next(b0)), R(b0), dr1);
                b1 = b2;
                b2 = next(b2);
                dot = 0.;
                for (uint32_t d = 0; d < n_d; ++d) dot += drL[d] * dr1[d];
                tot -= dot * i_4_lambda_tau / (window * path.tau);
            }
        }
        return tot;
    }

    // The walk of kinetic_class.h:112-119: from bead (p, b0) in steps of `skip` along the links until
    // bead_b = GetNextBead(b1 - b0) of the start; calls f(label, slice, next label, next slice) per link.
    template <class F>
    void Links(uint32_t p, uint32_t b0, uint32_t b1, uint32_t skip, F f) {
        const Mode m = path.mode;
        uint32_t end_b;
        const uint32_t end_p = path.Walk(*species, p, b0, b1 - b0, m, end_b);
        uint32_t ap = p, ab = species->bead_loop(b0 % species->n_bead), guard = 0;
        while (!(ap == end_p && ab == end_b)) {
            uint32_t nb;
            const uint32_t np_ = path.Walk(*species, ap, ab, skip, m, nb);
            f(ap, ab, np_, nb);
            ap = np_;
            ab = nb;
            if (++guard > species->n_part * species->n_bead) throw std::invalid_argument("segment end is not reachable at this level");
        }
    }

    // kinetic_class.h:105-122
    double GetAction(uint32_t b0, uint32_t b1, const Particles& parts, uint32_t level) override {
        uint32_t skip = 1u << level;
        double tot = 0., dr[3];
        for (auto& pr : parts) {
            if (pr.first != species->s_i) continue;
            Links(pr.second, b0, b1, skip, [&](uint32_t ap, uint32_t ab, uint32_t np_, uint32_t nb) {
                path.Dr(path.GetR(*species, ap, ab), path.GetR(*species, np_, nb), dr);
                tot -= rho_free_splines[skip - 1].GetLogRhoFree(dr, path.n_d);
            });
        }
        return tot;
    }

    // kinetic_class.h:125-144
    void GetActionGradient(uint32_t b0, uint32_t b1, const Particles& parts, uint32_t level, double* g) override {
        uint32_t skip = 1u << level;
        uint32_t n_d = path.n_d;
        double i4 = i_4_lambda_tau / skip;
        double tot[3] = {0., 0., 0.}, t[3];
        for (auto& pr : parts) {
            if (pr.first != species->s_i) continue;
            Links(pr.second, b0, b1, skip, [&](uint32_t ap, uint32_t ab, uint32_t np_, uint32_t nb) {
                uint32_t pb;
                const uint32_t pp = path.WalkBack(*species, ap, ab, skip, path.mode, pb);
                path.Dr(path.GetR(*species, pp, pb), path.GetR(*species, ap, ab), t);
                for (uint32_t d = 0; d < n_d; ++d) tot[d] -= t[d];
                path.Dr(path.GetR(*species, ap, ab), path.GetR(*species, np_, nb), t);
                for (uint32_t d = 0; d < n_d; ++d) tot[d] += t[d];
            });
        }
        for (uint32_t d = 0; d < n_d; ++d) g[d] = 2. * i4 * tot[d];
    }
};

// src/actions/single_action/trap_class.h:7-65
struct Trap : SingleAction {
    double omega, cofactor_a, cofactor_b;
    Trap(Path& p, const Input& in) : SingleAction(p, in) {
        omega = in.GetAttribute<double>("omega");
        cofactor_a = 0.5 * p.tau * omega * omega * (1. + p.tau * p.tau * omega * omega / 12.);
        cofactor_b = 0.5 * omega * omega * (1. + 3. * p.tau * p.tau * omega * omega / 12.);
    }
    double DActionDBeta() override {
        double tot = 0.;
        for (uint32_t p = 0; p < species->n_part; ++p)
            for (uint32_t b = 0; b < species->n_bead; ++b) {
                const double* r = path.GetR(*species, p, b);
                for (uint32_t d = 0; d < path.n_d; ++d) tot += r[d] * r[d];
            }
        return cofactor_b * tot;
    }
    double GetAction(uint32_t b0, uint32_t b1, const Particles& parts, uint32_t level) override {
        if (level > max_level) return 0.;
        bool check = false;
        for (auto& pr : parts)
            if (pr.first == species->s_i) check = true;
        if (!check) return 0.;
        uint32_t skip = 1u << level;
        double tot = 0.;
        for (auto& pr : parts)
            for (uint32_t b = b0; b < b1; b += skip) {
                const double* r = path.GetR(*species, pr.second, b);
                for (uint32_t d = 0; d < path.n_d; ++d) tot += r[d] * r[d];
            }
        return cofactor_a * skip * tot;
    }
};

// src/actions/pair_action/pair_action_class.h:12-420
struct PairAction : Action {
    bool is_constant, is_first_time = true, use_long_range;
    double dUdB_constant = 0., k_cut = 0., potential_constant = 0.;
    Species *species_a, *species_b;

    PairAction(Path& p, const Input& in) : Action(p, in) {
        species_a = &p.GetSpecies(in.GetAttribute<std::string>("species_a"));
        species_list.push_back(species_a->s_i);
        species_b = &p.GetSpecies(in.GetAttribute<std::string>("species_b"));
        species_list.push_back(species_b->s_i);
        use_long_range = in.GetAttribute<bool>("use_long_range", false);
        if (use_long_range) {
            if (!p.pbc) throw InputError("use_long_range needs periodic boundaries");
            k_cut = in.GetAttribute<double>("k_cut", p.ks.cutoff);
            p.ks.Setup(k_cut);
        }
        is_constant = (species_a == species_b) && (species_a->n_part == 1 || species_a->lambda == 0.);
    }

    virtual double CalcV(double r, double rp, uint32_t level) = 0;
    virtual double CalcVLong() = 0;
    virtual double CalcU(double r, double rp, double s, uint32_t level) = 0;
    virtual double CalcULong(uint32_t b0, uint32_t b1, uint32_t level) = 0;
    virtual double CalcdUdBeta(double r, double rp, double s, uint32_t level) = 0;
    virtual double CalcdUdBetaLong() = 0;

    static void SetLimits(double rmin, double rmax, double& r, double& rp) {
        if (r > rmax) r = rmax;
        else if (r < rmin) r = rmin;
        if (rp > rmax) rp = rmax;
        else if (rp < rmin) rp = rmin;
    }

    // pair_action_class.h:45-59
    std::vector<std::pair<uint32_t, uint32_t>> AllPairs() const {
        std::vector<std::pair<uint32_t, uint32_t>> pp;
        if (species_a == species_b) {
            for (uint32_t p = 0; p + 1 < species_a->n_part; ++p)
                for (uint32_t q = p + 1; q < species_b->n_part; ++q) pp.push_back({p, q});
        } else {
            for (uint32_t p = 0; p < species_a->n_part; ++p)
                for (uint32_t q = 0; q < species_b->n_part; ++q) pp.push_back({p, q});
        }
        return pp;
    }

    // pair_action_class.h:62-114
    void GenPairs(const Particles& parts, std::vector<uint32_t>& pa, std::vector<uint32_t>& pb, std::vector<std::pair<uint32_t, uint32_t>>& pp) {
        for (auto& pr : parts) {
            if (pr.first == species_a->s_i) pa.push_back(pr.second);
            else if (pr.first == species_b->s_i) pb.push_back(pr.second);
        }
        uint32_t n_a = (uint32_t)pa.size(), n_b = (uint32_t)pb.size();
        if (n_a == 0 && n_b == 0) return;
        std::vector<uint32_t> oa, ob;
        for (uint32_t i = 0; i < species_a->n_part; ++i)
            if (std::find(pa.begin(), pa.end(), i) == pa.end()) oa.push_back(i);
        for (uint32_t i = 0; i < species_b->n_part; ++i)
            if (std::find(pb.begin(), pb.end(), i) == pb.end()) ob.push_back(i);
        if (species_a == species_b) {
            for (auto p : pa)
                for (auto q : oa) pp.push_back({p, q});
            for (uint32_t p = 0; p + 1 < n_a; ++p)
                for (uint32_t q = p + 1; q < n_a; ++q) pp.push_back({pa[p], pa[q]});
        } else {
            for (auto p : pa)
                for (auto q : ob) pp.push_back({p, q});
            for (auto p : pb)
                for (auto q : oa) pp.push_back({q, p});
            for (auto p : pa)
                for (auto q : pb) pp.push_back({p, q});
        }
    }

    // pair_action_class.h:135-155 (central differences, eps = 1e-4)
    virtual void CalcGradientU(uint32_t bi, uint32_t bj, uint32_t pi, uint32_t pj, uint32_t level, double* tot) {
        double* rr = path.GetR(*species_a, pi, bi);
        double r0[3];
        for (uint32_t d = 0; d < path.n_d; ++d) r0[d] = rr[d];
        const double eps = 1.e-4;
        double a, b, c;
        for (uint32_t d = 0; d < path.n_d; ++d) {
            rr[d] = r0[d] + eps;
            path.DrDrpDrrp(bi, bj, *species_a, *species_b, pi, pj, a, b, c);
            double f1 = CalcU(a, b, c, level);
            rr[d] = r0[d] - eps;
            path.DrDrpDrrp(bi, bj, *species_a, *species_b, pi, pj, a, b, c);
            double f2 = CalcU(a, b, c, level);
            tot[d] = (f1 - f2) / (2. * eps);
            rr[d] = r0[d];
        }
    }
    virtual void CalcGradientULong(uint32_t, uint32_t, uint32_t, uint32_t, double* g) {
        for (uint32_t d = 0; d < path.n_d; ++d) g[d] = 0.;
    }

    // pair_action_class.h:241-264
    double DActionDBeta() override {
        if (is_constant && !is_first_time) return dUdB_constant;
        double tot = 0.;
        auto pp = AllPairs();
        for (size_t i = 0; i < pp.size(); ++i)
            for (uint32_t b = 0; b < species_a->n_bead; ++b) {
                double a, bb, c;
                path.DrDrpDrrp(b, b + 1, *species_a, *species_b, pp[i].first, pp[i].second, a, bb, c);
                tot += CalcdUdBeta(a, bb, c, 0);
            }
        if (use_long_range) tot += CalcdUdBetaLong();
        if (is_first_time) {
            is_first_time = false;
            dUdB_constant = tot;
        }
        return tot;
    }

    // pair_action_class.h:267-302
    double GetAction(uint32_t b0, uint32_t b1, const Particles& parts, uint32_t level) override {
        if (level > max_level || is_constant) return 0.;
        std::vector<uint32_t> pa, pb;
        std::vector<std::pair<uint32_t, uint32_t>> pp;
        GenPairs(parts, pa, pb, pp);
        if (pp.empty()) return 0.;
        uint32_t skip = 1u << level;
        double tot = 0.;
        for (uint32_t b = b0; b < b1; b += skip) {
            uint32_t bj = b + skip;
            for (auto& pr : pp) {
                double a, bb, c;
                path.DrDrpDrrp(b, bj, *species_a, *species_b, pr.first, pr.second, a, bb, c);
                tot += CalcU(a, bb, c, level);
            }
        }
        if (use_long_range) {
            if (species_a->need_update_rho_k && path.mode == NEW_MODE) path.UpdateRhoK(*species_a, b0, b1, pa, level);
            if (species_b->need_update_rho_k && path.mode == NEW_MODE) path.UpdateRhoK(*species_b, b0, b1, pb, level);
            tot += CalcULong(b0, b1, level);
        }
        return tot;
    }

    // pair_action_class.h:305-337
    void GetActionGradient(uint32_t b0, uint32_t b1, const Particles& parts, uint32_t level, double* g) override {
        for (uint32_t d = 0; d < path.n_d; ++d) g[d] = 0.;
        if (level > max_level || is_constant) return;
        std::vector<uint32_t> pa, pb;
        std::vector<std::pair<uint32_t, uint32_t>> pp;
        GenPairs(parts, pa, pb, pp);
        if (pp.empty()) return;
        uint32_t skip = 1u << level;
        double t[3];
        for (uint32_t b = b0; b < b1; b += skip) {
            uint32_t bj = b + skip;
            uint32_t bk = b - skip + species_a->n_bead;
            for (auto& pr : pp) {
                CalcGradientU(b, bj, pr.first, pr.second, level, t);
                for (uint32_t d = 0; d < path.n_d; ++d) g[d] += t[d];
                CalcGradientU(b, bk, pr.first, pr.second, level, t);
                for (uint32_t d = 0; d < path.n_d; ++d) g[d] += t[d];
            }
        }
        if (use_long_range) {
            for (auto& pr : pp) {
                CalcGradientULong(b0, b1, pr.first, level, t);
                for (uint32_t d = 0; d < path.n_d; ++d) g[d] += t[d];
            }
        }
    }

    // pair_action_class.h:369-395
    double Potential() override {
        if (is_constant && !is_first_time) return potential_constant;
        double tot = 0.;
        auto pp = AllPairs();
        double dr[3];
        for (size_t i = 0; i < pp.size(); ++i)
            for (uint32_t b = 0; b < species_a->n_bead; ++b) {
                path.Dr(path.GetR(*species_a, pp[i].first, b), path.GetR(*species_b, pp[i].second, b), dr);
                double rm = 0.;
                for (uint32_t d = 0; d < path.n_d; ++d) rm += dr[d] * dr[d];
                rm = std::sqrt(rm);
                path.Dr(path.GetR(*species_a, pp[i].first, b + 1), path.GetR(*species_b, pp[i].second, b + 1), dr);
                double rpm = 0.;
                for (uint32_t d = 0; d < path.n_d; ++d) rpm += dr[d] * dr[d];
                rpm = std::sqrt(rpm);
                tot += CalcV(rm, rpm, 0);
            }
        if (use_long_range) tot += CalcVLong();
        if (is_first_time) {
            is_first_time = false;
            potential_constant = tot;
        }
        return tot;
    }

    void Accept() override {
        if (use_long_range) {
            species_a->need_update_rho_k = true;
            species_b->need_update_rho_k = true;
        }
    }
    void Reject() override { Accept(); }
};

static bool fequal(double a, double b, double tol) { return std::fabs(a - b) < tol; }

// src/actions/pair_action/bare_pair_action_class.h:7-183
struct BarePairAction : PairAction {
    bool is_coulomb;
    double r_v_min, r_v_max, r_v_long_min = 0., r_v_long_max = 0., v_long_k_0 = 0., v_long_r_0 = 0.;
    Spline v_r_spline, v_long_r_spline;
    std::vector<double> v_long_k;

    BarePairAction(Path& p, const Input& in, const std::string& base_dir) : PairAction(p, in) {
        std::string file = in.GetAttribute<std::string>("file");
        if (!file.empty() && file[0] != '/' && !base_dir.empty()) file = base_dir + "/" + file;
        TableFile t = TableFile::Load(file);
        is_coulomb = in.GetAttribute<bool>("is_coulomb", false);
        const auto& r = t.Vec("v/diag/r");
        const auto& v = t.Vec("v/diag/v_r");
        if ((size_t)t.Scalar("v/diag/n_r") != r.size() || r.size() != v.size() || r.size() < 2)
            throw InputError("table '" + file + "': inconsistent v/diag grid");
        v_r_spline.Build(r, v, false);
        r_v_min = r.front();
        r_v_max = r.back();
        if (use_long_range) {
            const auto& rl = t.Vec("v/diag/r_long");
            const auto& vl = t.Vec("v/diag/v_long_r");
            v_long_r_0 = t.Scalar("v/diag/v_long_r_0");
            v_long_r_spline.Build(rl, vl, false);
            r_v_long_min = rl.front();
            r_v_long_max = rl.back();
            const auto& kv = t.Vec("v/diag/k");
            const auto& vk = t.Vec("v/diag/v_long_k");
            v_long_k_0 = t.Scalar("v/diag/v_long_k_0");
            v_long_k.assign(p.ks.K(), 0.);
            for (size_t k = 0; k < p.ks.K(); ++k)
                for (size_t j = 0; j < kv.size(); ++j)
                    if (fequal(p.ks.mags[k], kv[j], 1.e-8)) v_long_k[k] = vk[j];
        }
        if (species_a == species_b) {
            v_long_k_0 *= 0.5 * species_a->n_part * species_b->n_part * p.n_bead;
            v_long_r_0 *= -0.5 * species_a->n_part * p.n_bead;
        } else {
            v_long_k_0 *= species_a->n_part * species_b->n_part * p.n_bead;
            v_long_r_0 *= 0.;
        }
    }

    double CalcV(double r, double rp, uint32_t) override {
        SetLimits(r_v_min, r_v_max, r, rp);
        double v = 0.;
        if (is_coulomb) v += (0.5 / r) + (0.5 / rp);
        else v += 0.5 * v_r_spline.Eval(r) + 0.5 * v_r_spline.Eval(rp);
        if (use_long_range) {
            SetLimits(r_v_long_min, r_v_long_max, r, rp);
            v -= 0.5 * v_long_r_spline.Eval(r);
            v -= 0.5 * v_long_r_spline.Eval(rp);
        }
        return v;
    }

    double CalcVLong() override {
        const auto& ra = path.GetRhoK(*species_a);
        const auto& rb = path.GetRhoK(*species_b);
        size_t K = path.ks.K();
        double tot = 0.;
        for (size_t k = 0; k < K; ++k)
            for (uint32_t b = 0; b < path.n_bead; ++b) tot += CMag2(ra[(size_t)b * K + k], rb[(size_t)b * K + k]) * v_long_k[k];
        if (species_a != species_b) tot *= 2.;
        return tot + v_long_k_0 + v_long_r_0;
    }

    double CalcU(double r, double rp, double, uint32_t level) override {
        uint32_t skip = 1u >> level;  // bare_pair_action_class.h:147 (sic)
        double level_tau = skip * path.tau;
        return level_tau * CalcV(r, rp, level);
    }

    double CalcULong(uint32_t b0, uint32_t b1, uint32_t level) override {
        const auto& ra = path.GetRhoK(*species_a);
        const auto& rb = path.GetRhoK(*species_b);
        size_t K = path.ks.K();
        uint32_t skip = 1u << level;
        double tot = 0.;
        for (size_t k = 0; k < K; ++k)
            for (uint32_t b = b0; b < b1; b += skip)
                tot += v_long_k[k] * CMag2(ra[(size_t)species_a->bead_loop(b) * K + k], rb[(size_t)species_b->bead_loop(b) * K + k]);
        if (species_a != species_b) tot *= 2.;
        return skip * path.tau * tot;
    }

    double CalcdUdBeta(double r, double rp, double, uint32_t level) override { return CalcV(r, rp, level); }
    double CalcdUdBetaLong() override { return CalcVLong(); }
};

// src/actions/pair_action/ilkka_pair_action_class.h:7-433
struct IlkkaPairAction : PairAction {
    double r_u_min = 0., r_u_max = 0., r_du_min = 0., r_du_max = 0., r_v_min = 0., r_v_max = 0.;
    double r_v_long_min = 0., r_v_long_max = 0.;
    double du_long_k_0 = 0., du_long_r_0 = 0., v_long_k_0 = 0., v_long_r_0 = 0.;
    std::vector<double> u_long_k, du_long_k, v_long_k;
    Spline u_long_r_spline, du_long_r_spline, v_r_spline, v_long_r_spline;
    Spline2 u_xy_spline, du_xy_spline;

    // The k-space datasets hold one value per distinct |k|; each stored k-vector takes the value
    // of its magnitude (ilkka_pair_action_class.h:308-315).
    static std::vector<double> ByMagnitude(const Path& p, const std::vector<double>& kv, const std::vector<double>& vals) {
        std::vector<double> out(p.ks.K(), 0.);
        for (size_t k = 0; k < p.ks.K(); ++k)
            for (size_t j = 0; j < kv.size(); ++j)
                if (fequal(p.ks.mags[k], kv[j], 1.e-8)) out[k] = vals[j];
        return out;
    }

    IlkkaPairAction(Path& p, const Input& in, const std::string& base_dir) : PairAction(p, in) {
        std::string file = in.GetAttribute<std::string>("file");
        if (!file.empty() && file[0] != '/' && !base_dir.empty()) file = base_dir + "/" + file;
        TableFile t = TableFile::Load(file);
        auto grid2 = [&](const std::string& g, const std::string& f, Spline2& sp) {
            const auto& x = t.Vec(g + "/off_diag/x");
            const auto& y = t.Vec(g + "/off_diag/y");
            if ((size_t)t.Scalar(g + "/off_diag/n_x") != x.size() || (size_t)t.Scalar(g + "/off_diag/n_y") != y.size())
                throw InputError("table '" + file + "': inconsistent " + g + "/off_diag grid");
            sp.Build(x, y, t.Vec(g + "/off_diag/" + f));
        };
        grid2("u", "u_xy", u_xy_spline);  // :266-280
        if (use_long_range) {             // :282-316
            const auto& r = t.Vec("u/diag/r_long");
            u_long_r_spline.Build(r, t.Vec("u/diag/u_long_r"), false);
            r_u_min = r.front();
            r_u_max = r.back();
            u_long_k = ByMagnitude(p, t.Vec("u/diag/k"), t.Vec("u/diag/u_long_k"));
        }
        grid2("du", "du_xy", du_xy_spline);  // :318-332
        if (use_long_range) {                // :334-368
            const auto& r = t.Vec("du/diag/r_long");
            du_long_r_spline.Build(r, t.Vec("du/diag/du_long_r"), false);
            du_long_r_0 = t.Scalar("du/diag/du_long_r_0");
            r_du_min = r.front();
            r_du_max = r.back();
            du_long_k = ByMagnitude(p, t.Vec("du/diag/k"), t.Vec("du/diag/du_long_k"));
            du_long_k_0 = t.Scalar("du/diag/du_long_k_0");
        }
        {  // :370-382
            const auto& r = t.Vec("v/diag/r");
            v_r_spline.Build(r, t.Vec("v/diag/v_r"), false);
            r_v_min = r.front();
            r_v_max = r.back();
        }
        if (use_long_range) {  // :384-418
            const auto& r = t.Vec("v/diag/r_long");
            v_long_r_spline.Build(r, t.Vec("v/diag/v_long_r"), false);
            v_long_r_0 = t.Scalar("v/diag/v_long_r_0");
            r_v_long_min = r.front();
            r_v_long_max = r.back();
            v_long_k = ByMagnitude(p, t.Vec("v/diag/k"), t.Vec("v/diag/v_long_k"));
            v_long_k_0 = t.Scalar("v/diag/v_long_k_0");
        }
        if (species_a == species_b) {  // :420-431
            du_long_k_0 *= 0.5 * species_a->n_part * species_b->n_part * p.n_bead;
            du_long_r_0 *= -0.5 * species_a->n_part * p.n_bead;
            v_long_k_0 *= 0.5 * species_a->n_part * species_b->n_part * p.n_bead;
            v_long_r_0 *= -0.5 * species_a->n_part * p.n_bead;
        } else {
            du_long_k_0 *= species_a->n_part * species_b->n_part * p.n_bead;
            du_long_r_0 *= 0.;
            v_long_k_0 *= species_a->n_part * species_b->n_part * p.n_bead;
            v_long_r_0 *= 0.;
        }
    }

    // Sum over stored k of coef_k Re(rho_a conj rho_b) over slices [b0, b1) at stride skip, x2 for
    // two species (:104-122, :151-169).
    double KSum(const std::vector<double>& coef, uint32_t b0, uint32_t b1, uint32_t skip) {
        const auto& ra = path.GetRhoK(*species_a);
        const auto& rb = path.GetRhoK(*species_b);
        size_t K = path.ks.K();
        double tot = 0.;
        for (size_t k = 0; k < K; ++k)
            for (uint32_t b = b0; b < b1; b += skip)
                tot += coef[k] * CMag2(ra[(size_t)species_a->bead_loop(b) * K + k], rb[(size_t)species_b->bead_loop(b) * K + k]);
        if (species_a != species_b) tot *= 2.;
        return tot;
    }

    double CalcV(double r, double rp, uint32_t) override {  // :34-54
        SetLimits(r_v_min, r_v_max, r, rp);
        double v = 0.5 * v_r_spline.Eval(r) + 0.5 * v_r_spline.Eval(rp);
        if (use_long_range) {
            SetLimits(r_v_long_min, r_v_long_max, r, rp);
            v -= 0.5 * v_long_r_spline.Eval(r);
            v -= 0.5 * v_long_r_spline.Eval(rp);
        }
        return v;
    }
    double CalcVLong() override {  // :57-74 (summed in k-major order as the reference's loop)
        const auto& ra = path.GetRhoK(*species_a);
        const auto& rb = path.GetRhoK(*species_b);
        size_t K = path.ks.K();
        double tot = 0.;
        for (size_t k = 0; k < K; ++k)
            for (uint32_t b = 0; b < path.n_bead; ++b) tot += v_long_k[k] * CMag2(ra[(size_t)b * K + k], rb[(size_t)b * K + k]);
        if (species_a != species_b) tot *= 2.;
        return tot + v_long_k_0 + v_long_r_0;
    }
    double CalcU(double r, double rp, double s, uint32_t) override {  // :77-101
        double q = 0.5 * (r + rp);
        double u = u_xy_spline.Eval(q + 0.5 * s, q - 0.5 * s);
        if (use_long_range) {
            SetLimits(r_u_min, r_u_max, r, rp);
            u -= 0.5 * u_long_r_spline.Eval(r);
            u -= 0.5 * u_long_r_spline.Eval(rp);
        }
        return u;
    }
    double CalcULong(uint32_t b0, uint32_t b1, uint32_t level) override { return KSum(u_long_k, b0, b1, 1u << level); }  // :104-122
    double CalcdUdBeta(double r, double rp, double s, uint32_t) override {  // :125-149
        double q = 0.5 * (r + rp);
        double du = du_xy_spline.Eval(q + 0.5 * s, q - 0.5 * s);
        if (use_long_range) {
            SetLimits(r_du_min, r_du_max, r, rp);
            du -= 0.5 * du_long_r_spline.Eval(r);
            du -= 0.5 * du_long_r_spline.Eval(rp);
        }
        return du;
    }
    double CalcdUdBetaLong() override { return KSum(du_long_k, 0, path.n_bead, 1) + du_long_k_0 + du_long_r_0; }  // :152-169

    // :172-222, the chain rule through (x, y); r is the vector of DrDrpDrrp (second minus first particle).
    void CalcGradientU(uint32_t bi, uint32_t bj, uint32_t pi, uint32_t pj, uint32_t, double* tot) override {
        const uint32_t nd = path.n_d;
        double rv[3], rp[3], rrp[3];
        const double* a0 = path.GetR(*species_b, pj, bi);
        const double* c0 = path.GetR(*species_a, pi, bi);
        const double* a1 = path.GetR(*species_b, pj, bj);
        const double* c1 = path.GetR(*species_a, pi, bj);
        for (uint32_t d = 0; d < nd; ++d) {
            rv[d] = a0[d] - c0[d];
            rp[d] = a1[d] - c1[d];
        }
        for (uint32_t d = 0; d < nd; ++d) {
            rv[d] -= std::nearbyint(rv[d] * path.iL) * path.L;
            rp[d] += std::nearbyint((rv[d] - rp[d]) * path.iL) * path.L;
        }
        for (uint32_t d = 0; d < nd; ++d) rrp[d] = rv[d] - rp[d];
        for (uint32_t d = 0; d < nd; ++d) rrp[d] -= std::nearbyint(rrp[d] * path.iL) * path.L;
        double a = 0., b = 0., c = 0.;
        for (uint32_t d = 0; d < nd; ++d) {
            a += rv[d] * rv[d];
            b += rp[d] * rp[d];
            c += rrp[d] * rrp[d];
        }
        double r_mag = std::sqrt(a), r_p_mag = std::sqrt(b), s_mag = std::sqrt(c);
        double q = 0.5 * (r_mag + r_p_mag);
        double u, du_dx, du_dy;
        u_xy_spline.EvalVG(q + 0.5 * s_mag, q - 0.5 * s_mag, u, du_dx, du_dy);
        double rh[3], sh[3];
        for (uint32_t d = 0; d < nd; ++d) {
            rh[d] = r_mag == 0. ? 0. : rv[d] / r_mag;
            sh[d] = s_mag == 0. ? 0. : rrp[d] / s_mag;
        }
        for (uint32_t d = 0; d < nd; ++d) tot[d] = -0.5 * (du_dx * (rh[d] + sh[d]) + du_dy * (rh[d] - sh[d]));
        if (use_long_range) {
            SetLimits(r_u_min, r_u_max, r_mag, r_p_mag);
            double tu, tdu;
            u_long_r_spline.EvalVG(r_mag, tu, tdu);
            for (uint32_t d = 0; d < nd; ++d) tot[d] -= 0.5 * tdu * rh[d];
        }
    }

    // :231-249: per-bead densities of p_i (current mode) against species b's slice densities.
    void CalcGradientULong(uint32_t b0, uint32_t b1, uint32_t pi, uint32_t level, double* g) override {
        const auto& rb = path.GetRhoK(*species_b);
        size_t K = path.ks.K();
        uint32_t skip = 1u << level;
        double tot[3] = {0., 0., 0.};
        std::vector<cplx> tmp;
        for (uint32_t b = b0; b < b1; b += skip) {
            const cplx* ri = path.BeadRhoK(*species_a, pi, b, path.mode, &tmp);
            for (size_t k = 0; k < K; ++k) {
                const cplx& rbk = rb[(size_t)species_b->bead_loop(b) * K + k];
                double f = u_long_k[k] * (ri[k].real() * rbk.imag() - ri[k].imag() * rbk.real());
                for (uint32_t d = 0; d < path.n_d; ++d) tot[d] += f * path.ks.vecs[k][d];
            }
        }
        if (species_a != species_b)
            for (uint32_t d = 0; d < path.n_d; ++d) tot[d] *= 2.;
        for (uint32_t d = 0; d < path.n_d; ++d) g[d] = tot[d];
    }
};

// src/actions/pair_action/david_pair_action_class.h:7-361. The squarer's expansion
//   U = (u_00(r) + u_00(r'))/2 + sum_{k=1..n} sum_{j=0..k} u_kj(q) z^(2j) s^(2(k-j)),
// q = (r + r')/2, z = r - r', on one radial grid; component 0 of every multi-spline is the potential.
// One table per level up to max_level (n_tau = max_level + 1); level l reads table l (u_kj(level)).
struct DavidPairAction : PairAction {
    uint32_t n_order = 0, n_val = 0;
    double r_min = 0., r_max = 0.;
    double du_long_k_0 = 0., du_long_r_0 = 0., v_long_k_0 = 0., v_long_r_0 = 0.;
    std::vector<double> u_long_k, du_long_k, v_long_k;
    std::vector<std::vector<Spline>> u_kj, du_kj;  // [level][n_val + 1 components]

    DavidPairAction(Path& p, const Input& in, const std::string& base_dir) : PairAction(p, in) {
        n_order = in.GetAttribute<uint32_t>("n_order", 0);  // pair_action_class.h:208
        std::string file = in.GetAttribute<std::string>("file");
        if (!file.empty() && file[0] != '/' && !base_dir.empty()) file = base_dir + "/" + file;
        TableFile t = TableFile::Load(file);
        const std::string pre = "u_kj_" + std::to_string(n_order), dpre = "du_kj_dbeta_" + std::to_string(n_order);
        const auto& grid = t.Vec(pre + "/grid/grid_points");  // :211-232 (a general grid)
        const size_t n_grid = grid.size();
        if ((size_t)t.Scalar(pre + "/grid/n_grid_points") != n_grid || n_grid < 2)
            throw InputError("table '" + file + "': inconsistent grid");
        r_min = grid.front();
        r_max = grid.back();
        const size_t n_tau = (size_t)max_level + 1;  // :234-246
        const auto& taus = t.Vec(pre + "/taus");
        if (taus.size() < n_tau) throw InputError("table '" + file + "': fewer taus than max_level + 1");
        bool found = false;
        for (size_t i = 0; i < n_tau; ++i) found |= std::fabs(taus[i] - p.tau) < 1.0e-6;
        if (!found) throw InputError("table '" + file + "': tau of the path not found");
        const auto& V = t.Vec("potential/data");
        n_val = 1;
        for (uint32_t i = 1; i <= n_order; ++i) n_val += 1 + i;  // :252-255
        auto load = [&](const std::string& key, std::vector<std::vector<Spline>>& out) {  // :257-316
            const auto& d = t.Vec(key);  // n_val x n_grid x n_tau, value index fastest
            if (d.size() < (size_t)n_val * n_grid * n_tau || V.size() != n_grid) throw InputError("table '" + file + "': short " + key);
            out.assign(n_tau, std::vector<Spline>(n_val + 1));
            std::vector<double> col(n_grid);
            // :262-271 fill the grid points below the last one only (the zeroing of the last one is
            // commented out); the zero-initialised arrays leave zero there for every component.
            for (size_t l = 0; l < n_tau; ++l)
                for (uint32_t v = 0; v <= n_val; ++v) {
                    for (size_t g = 0; g < n_grid; ++g)
                        col[g] = g + 1 == n_grid ? 0. : v == 0 ? V[g] : d[(v - 1) + g * n_val + l * n_val * n_grid];
                    out[l][v].Build(grid, col, false);
                }
        };
        load(pre + "/data", u_kj);
        load(dpre + "/data", du_kj);
        if (use_long_range) {  // :318-357
            const auto& kv = t.Vec("long_range/k_points");
            const auto& uk = t.Vec("long_range/u_k");
            const double vol = p.vol;
            u_long_k.assign(p.ks.K(), 0.);
            du_long_k.assign(p.ks.K(), 0.);
            v_long_k.assign(p.ks.K(), 0.);
            for (size_t i = 0; i < kv.size(); ++i) {
                const double vk = uk[i] / vol;
                if (fequal(0., kv[i], 1.e-8)) v_long_k_0 = vk;
                for (size_t k = 0; k < p.ks.K(); ++k)
                    if (fequal(p.ks.mags[k], kv[i], 1.e-8)) {
                        u_long_k[k] = vk * p.tau;
                        du_long_k[k] = vk;
                        v_long_k[k] = vk;
                    }
            }
            v_long_r_0 = t.Scalar("squarer/v_image");
            du_long_r_0 = v_long_r_0;
            du_long_k_0 = v_long_k_0;
            if (species_a == species_b) {
                du_long_k_0 *= 0.5 * species_a->n_part * species_b->n_part * p.n_bead;
                du_long_r_0 *= -0.5 * species_a->n_part * p.n_bead;
                v_long_k_0 *= 0.5 * species_a->n_part * species_b->n_part * p.n_bead;
                v_long_r_0 *= -0.5 * species_a->n_part * p.n_bead;
            } else {
                du_long_k_0 *= species_a->n_part * species_b->n_part * p.n_bead;
                du_long_r_0 *= 0.;
                v_long_k_0 *= species_a->n_part * species_b->n_part * p.n_bead;
                v_long_r_0 *= 0.;
            }
        }
    }

    double KSum(const std::vector<double>& coef, uint32_t b0, uint32_t b1, uint32_t skip) {
        const auto& ra = path.GetRhoK(*species_a);
        const auto& rb = path.GetRhoK(*species_b);
        size_t K = path.ks.K();
        double tot = 0.;
        for (size_t k = 0; k < K; ++k)
            for (uint32_t b = b0; b < b1; b += skip)
                tot += coef[k] * CMag2(ra[(size_t)species_a->bead_loop(b) * K + k], rb[(size_t)species_b->bead_loop(b) * K + k]);
        if (species_a != species_b) tot *= 2.;
        return tot;
    }

    // Off-diagonal sum of the expansion at q with the coefficients of `comp` (:80-99, :146-163).
    double OffDiagonal(const std::vector<Spline>& comp, double q, double z, double s) const {
        double z2 = z * z, s2 = s * s, is2 = 1. / s2, s2k = s2, tot = 0.;
        for (uint32_t k = 1; k <= n_order; ++k) {
            double z2j = 1., cs = s2k;
            for (uint32_t j = 0; j <= k; ++j) {
                tot += comp[k * (k + 1) / 2 + j + 1].Eval(q) * z2j * cs;
                z2j *= z2;
                cs *= is2;
            }
            s2k *= s2;
        }
        return tot;
    }

    double CalcV(double r, double rp, uint32_t level) override {  // :34-47
        SetLimits(r_min, r_max, r, rp);
        return 0.5 * (u_kj[level][0].Eval(r) + u_kj[level][0].Eval(rp));
    }
    double CalcVLong() override { return KSum(v_long_k, 0, path.n_bead, 1) + v_long_k_0 + v_long_r_0; }  // :50-66
    double CalcU(double r, double rp, double s, uint32_t level) override {  // :69-102
        double q = 0.5 * (r + rp), z = r - rp;
        SetLimits(r_min, r_max, r, rp);
        const auto& t = u_kj[level];
        double u = 0.5 * (t[1].Eval(r) + t[1].Eval(rp));
        if (s > 0.0 && q < r_max) u += OffDiagonal(t, q, z, s);
        return u;
    }
    double CalcULong(uint32_t b0, uint32_t b1, uint32_t level) override { return KSum(u_long_k, b0, b1, 1u << level); }  // :105-123
    double CalcdUdBeta(double r, double rp, double s, uint32_t level) override {  // :126-167
        double q = 0.5 * (r + rp), z = r - rp;
        SetLimits(r_min, r_max, r, rp);
        const auto& t = du_kj[level];
        double v = 0.5 * (t[0].Eval(r) + t[0].Eval(rp));
        double du = 0.5 * (t[1].Eval(r) + t[1].Eval(rp)) + v;
        if (s > 0.0 && q < r_max) du += OffDiagonal(t, q, z, s);
        return du;
    }
    double CalcdUdBetaLong() override { return KSum(du_long_k, 0, path.n_bead, 1) + du_long_k_0 + du_long_r_0; }  // :170-186
};

// ---------------------------------------------------------------------------------------------
// Moves: Bisect (src/events/moves/single_species_move/bisect/bisect_class.h:8-214).
// ---------------------------------------------------------------------------------------------
// Whole-ring action at level 0 and its exact gradient (checker for the library's
// pimc_total_action / pimc_action_gradient_path and the HMC move built on them). Definitions:
//   Kinetic  sum_{p,b} -log rho_free(r_{p,b+1} - r_{p,b})        (kinetic_class.h:105-122)
//   Trap     cofactor_a sum_{p,b} |r_{p,b}|^2                       (trap_class.h:40-62)
//   Bare     tau sum_pairs sum_b V(|d_b|), d_b the minimum image of r_q - r_p on slice b, V the
//            clamped per-bead potential of CalcV (bare_pair_action_class.h:98-111), plus the Ewald
//            sum tau sum_b sum_k v_k Re(rho_a conj(rho_b)) (x2 for a != b, bare_pair_action_class.h:152-165)
// The gradient is the analytic derivative of each term.
static bool SelectedAction(const Action& a, int sel, int i) {
    if (a.is_importance_weight) return false;
    if (sel >= 0) return sel == i;
    if (sel == -2) return a.type != "Kinetic";
    return true;
}

static const double* RAt(const Path& path, const double* R, uint32_t g, uint32_t b) {
    return R + ((size_t)g * path.n_bead + (b % path.n_bead)) * path.n_d;
}

static void WholeRho(Path& path, const double* R, std::vector<std::vector<cplx>>& rho) {
    const size_t K = path.ks.K();
    rho.assign(path.species.size(), {});
    if (!K) return;
    for (auto& s : path.species) {
        auto& out = rho[s.s_i];
        out.assign((size_t)path.n_bead * K, cplx(0., 0.));
        for (uint32_t b = 0; b < path.n_bead; ++b)
            for (uint32_t p = 0; p < s.n_part; ++p) {
                path.ks.CalcC(RAt(path, R, s.offset + p, b));
                for (size_t k = 0; k < K; ++k) {
                    cplx f = 1.;
                    for (uint32_t d = 0; d < path.n_d; ++d) f *= path.ks.c_k[d][path.ks.indices[k][d]];
                    out[(size_t)b * K + k] += f;
                }
            }
    }
}

// Value and slope of a spline, zero slope outside its grid (where Eval holds the end value).
static void SplineVG(const Spline& sp, double t, double& v, double& g) {
    const bool in = t >= sp.x.front() && t <= sp.x.back();
    sp.EvalVG(t, v, g);
    if (!in) g = 0.;
}

static void KineticTerms(Kinetic& k, double* d, uint32_t nd, double& phi, double* dphi) {
    const FreeSpline& fs = k.rho_free_splines[0];
    phi = 0.;
    for (uint32_t c = 0; c < nd; ++c) {
        double v = 0., g = 0.;
        if (k.n_images > 0) SplineVG(fs.image_action, d[c], v, g);
        phi += v + d[c] * d[c] * fs.i_4_lambda_tau;
        dphi[c] = g + 2. * d[c] * fs.i_4_lambda_tau;
    }
}

static void BareVBead(const BarePairAction& a, double r, double& v, double& dv) {
    const bool in1 = r >= a.r_v_min && r <= a.r_v_max;
    const double r1 = std::min(std::max(r, a.r_v_min), a.r_v_max);
    if (a.is_coulomb) {
        v = 1. / r1;
        dv = in1 ? -1. / (r1 * r1) : 0.;
    } else {
        double g;
        a.v_r_spline.EvalVG(r1, v, g);
        dv = in1 ? g : 0.;
    }
    if (a.use_long_range) {
        const bool in2 = r1 >= a.r_v_long_min && r1 <= a.r_v_long_max;
        const double r2 = std::min(std::max(r1, a.r_v_long_min), a.r_v_long_max);
        double vl, gl;
        a.v_long_r_spline.EvalVG(r2, vl, gl);
        v -= vl;
        if (in1 && in2) dv -= gl;
    }
}

static double WholeAction(Path& path, std::vector<std::unique_ptr<Action>>& actions, int sel, const double* R) {
    const uint32_t M = path.n_bead, nd = path.n_d;
    std::vector<std::vector<cplx>> rho;
    bool have_rho = false;
    double total = 0.;
    for (size_t i = 0; i < actions.size(); ++i) {
        Action* a = actions[i].get();
        if (!SelectedAction(*a, sel, (int)i)) continue;
        if (auto* k = dynamic_cast<Kinetic*>(a)) {
            const Species& s = *k->species;
            for (uint32_t p = 0; p < s.n_part; ++p)
                for (uint32_t b = 0; b < M; ++b) {
                    double d[3], dphi[3], phi;
                    path.Dr(RAt(path, R, s.offset + p, b + 1), RAt(path, R, s.offset + p, b), d);
                    KineticTerms(*k, d, nd, phi, dphi);
                    total += phi;
                }
        } else if (auto* t = dynamic_cast<Trap*>(a)) {
            const Species& s = *t->species;
            for (uint32_t p = 0; p < s.n_part; ++p)
                for (uint32_t b = 0; b < M; ++b) {
                    const double* r = RAt(path, R, s.offset + p, b);
                    double r2 = 0.;
                    for (uint32_t c = 0; c < nd; ++c) r2 += r[c] * r[c];
                    total += t->cofactor_a * r2;
                }
        } else if (dynamic_cast<IlkkaPairAction*>(a) || dynamic_cast<DavidPairAction*>(a)) {
            throw InputError("the whole-ring action covers Kinetic, HarmonicTrap and BarePairAction");
        } else if (auto* bp = dynamic_cast<BarePairAction*>(a)) {
            if (bp->is_constant) continue;
            for (auto& pr : bp->AllPairs()) {
                const uint32_t ga = bp->species_a->offset + pr.first, gb = bp->species_b->offset + pr.second;
                for (uint32_t b = 0; b < M; ++b) {
                    double d[3], r2 = 0., v, dv;
                    path.Dr(RAt(path, R, gb, b), RAt(path, R, ga, b), d);
                    for (uint32_t c = 0; c < nd; ++c) r2 += d[c] * d[c];
                    BareVBead(*bp, std::sqrt(r2), v, dv);
                    total += path.tau * v;
                }
            }
            if (bp->use_long_range) {
                if (!have_rho) {
                    WholeRho(path, R, rho);
                    have_rho = true;
                }
                const auto& ra = rho[bp->species_a->s_i];
                const auto& rb = rho[bp->species_b->s_i];
                const size_t K = path.ks.K();
                double lr = 0.;
                for (uint32_t b = 0; b < M; ++b)
                    for (size_t k = 0; k < K; ++k) lr += bp->v_long_k[k] * CMag2(ra[(size_t)b * K + k], rb[(size_t)b * K + k]);
                total += (bp->species_a == bp->species_b ? 1. : 2.) * path.tau * lr;
            }
        }
    }
    return total;
}

static void WholeGradient(Path& path, std::vector<std::unique_ptr<Action>>& actions, int sel, const double* R, double* G) {
    const uint32_t M = path.n_bead, nd = path.n_d;
    std::fill(G, G + (size_t)path.n_total * M * nd, 0.);
    auto gat = [&](uint32_t g, uint32_t b) { return G + ((size_t)g * M + (b % M)) * nd; };
    std::vector<std::vector<cplx>> rho;
    bool have_rho = false;
    for (size_t i = 0; i < actions.size(); ++i) {
        Action* a = actions[i].get();
        if (!SelectedAction(*a, sel, (int)i)) continue;
        if (auto* k = dynamic_cast<Kinetic*>(a)) {
            const Species& s = *k->species;
            for (uint32_t p = 0; p < s.n_part; ++p)
                for (uint32_t b = 0; b < M; ++b) {
                    const uint32_t g = s.offset + p;
                    double d[3], dphi[3], phi;
                    path.Dr(RAt(path, R, g, b + 1), RAt(path, R, g, b), d);  // link b -> b+1
                    KineticTerms(*k, d, nd, phi, dphi);
                    for (uint32_t c = 0; c < nd; ++c) {
                        gat(g, b + 1)[c] += dphi[c];
                        gat(g, b)[c] -= dphi[c];
                    }
                }
        } else if (auto* t = dynamic_cast<Trap*>(a)) {
            const Species& s = *t->species;
            for (uint32_t p = 0; p < s.n_part; ++p)
                for (uint32_t b = 0; b < M; ++b) {
                    const double* r = RAt(path, R, s.offset + p, b);
                    for (uint32_t c = 0; c < nd; ++c) gat(s.offset + p, b)[c] += 2. * t->cofactor_a * r[c];
                }
        } else if (dynamic_cast<IlkkaPairAction*>(a) || dynamic_cast<DavidPairAction*>(a)) {
            throw InputError("the whole-ring gradient covers Kinetic, HarmonicTrap and BarePairAction");
        } else if (auto* bp = dynamic_cast<BarePairAction*>(a)) {
            if (bp->is_constant) continue;
            for (auto& pr : bp->AllPairs()) {
                const uint32_t ga = bp->species_a->offset + pr.first, gb = bp->species_b->offset + pr.second;
                for (uint32_t b = 0; b < M; ++b) {
                    double d[3], r2 = 0., v, dv;
                    path.Dr(RAt(path, R, ga, b), RAt(path, R, gb, b), d);  // r_a - r_b
                    for (uint32_t c = 0; c < nd; ++c) r2 += d[c] * d[c];
                    const double r = std::sqrt(r2);
                    BareVBead(*bp, r, v, dv);
                    if (r > 0.)
                        for (uint32_t c = 0; c < nd; ++c) {
                            const double f = path.tau * dv * d[c] / r;
                            gat(ga, b)[c] += f;
                            gat(gb, b)[c] -= f;
                        }
                }
            }
            if (bp->use_long_range) {
                if (!have_rho) {
                    WholeRho(path, R, rho);
                    have_rho = true;
                }
                const size_t K = path.ks.K();
                auto force = [&](const Species& s, const std::vector<cplx>& other) {
                    for (uint32_t p = 0; p < s.n_part; ++p)
                        for (uint32_t b = 0; b < M; ++b) {
                            path.ks.CalcC(RAt(path, R, s.offset + p, b));
                            double acc[3] = {0., 0., 0.};
                            for (size_t k = 0; k < K; ++k) {
                                cplx e = 1.;
                                for (uint32_t c = 0; c < nd; ++c) e *= path.ks.c_k[c][path.ks.indices[k][c]];
                                const double f = bp->v_long_k[k] * std::imag(std::conj(other[(size_t)b * K + k]) * e);
                                for (uint32_t c = 0; c < nd; ++c) acc[c] += f * path.ks.vecs[k][c];
                            }
                            for (uint32_t c = 0; c < nd; ++c) gat(s.offset + p, b)[c] += -2. * path.tau * acc[c];
                        }
                };
                const Species& sa = *bp->species_a;
                const Species& sb = *bp->species_b;
                force(sa, rho[sb.s_i]);
                if (&sa != &sb) force(sb, rho[sa.s_i]);
            }
        }
    }
}

struct Move {
    std::string name, type;
    uint64_t n_accept = 0, n_attempt = 0;
    uint64_t attempt_counter = 0;
    virtual ~Move() {}
    virtual bool Attempt() = 0;
    virtual void Accept() = 0;
    virtual void Reject() = 0;
    virtual void ResetBlock() {}
    void DoEvent() {
        n_attempt++;
        if (Attempt()) {
            n_accept++;
            Accept();
        } else
            Reject();
        attempt_counter++;
    }
};

struct Bisect : Move {
    Path& path;
    Species* species;
    std::vector<Action*> action_list;
    uint32_t n_level, n_bisect_beads, bead0 = 0, bead1 = 0, move_index, seed, chain;
    int n_images;
    bool adaptive;
    double target_ratio = 0., i_4_lambda_tau;
    bool first_block = true;
    std::vector<FreeSpline> rho_free_splines;
    std::vector<std::pair<uint32_t, uint32_t>> affected;  // (particle, bead) in species

    Bisect(Path& p, std::vector<std::unique_ptr<Action>>& actions, const Input& in, uint32_t idx, uint32_t sd, uint32_t ch)
        : path(p), move_index(idx), seed(sd), chain(ch) {
        name = in.GetAttribute<std::string>("name");
        type = in.GetAttribute<std::string>("type");
        species = &p.GetSpecies(in.GetAttribute<std::string>("species"));
        i_4_lambda_tau = 1. / (4. * species->lambda * p.tau);
        for (auto& a : actions)  // move_class.h:27-31
            if (std::find(a->species_list.begin(), a->species_list.end(), species->s_i) != a->species_list.end())
                action_list.push_back(a.get());
        n_level = in.GetAttribute<uint32_t>("n_level");
        n_images = in.GetAttribute<int>("n_images", 0);
        adaptive = in.GetAttribute<bool>("adaptive", false);
        if (adaptive) target_ratio = in.GetAttribute<double>("target_ratio");
        n_bisect_beads = 1u << n_level;
        if (n_bisect_beads > species->n_bead) throw InputError("bisection segment longer than the path");
        uint32_t n_spline = (uint32_t)std::floor(std::log2((double)species->n_bead));
        for (uint32_t i = 0; i < n_spline; ++i)
            rho_free_splines.emplace_back(p.L, n_images, species->lambda, 0.5 * p.tau * (1u << i), false);
    }

    // bisect_class.h:142-155
    void ResetBlock() override {
        if (!first_block && adaptive && n_attempt > 0) {
            double ratio = (double)n_accept / (double)n_attempt;
            if (ratio < target_ratio && n_level > 1) n_level--;
            else if ((1u << n_level) < species->n_bead / 2) n_level++;
            n_bisect_beads = 1u << n_level;
        }
        first_block = false;
        n_accept = 0;
        n_attempt = 0;
    }

    // Sampling of one bisection level along beads lab/sl[0..B] (NEW links) for the bisection, with the
    // OLD-mode neighbours of the last midpoint taken from old_end (bisect_class.h:74-94,
    // perm_bisect_iterative_class.h:167-192): accumulates both log sampling probabilities.
    void SampleLevel(const Stream& st, uint32_t& mid_counter, uint32_t block_base, int level_i, const std::vector<uint32_t>& lab,
                     const std::vector<uint32_t>& sl, uint32_t old_end_p, uint32_t old_end_b, double& old_lsp, double& new_lsp) {
        const uint32_t skip = 1u << level_i, n_d = path.n_d;
        const double sigma = std::sqrt(species->lambda * path.tau * skip);
        for (uint32_t a = 0; a < n_bisect_beads; a += 2 * skip) {
            const uint32_t b = a + skip, c = a + 2 * skip;
            double rbar[3], delta[3], t[3];
            {
                const uint32_t cp = c == n_bisect_beads ? old_end_p : lab[c], cb = c == n_bisect_beads ? old_end_b : sl[c];
                const double* ra = path.GetRMode(*species, lab[a], sl[a], OLD_MODE);
                const double* rc = path.GetRMode(*species, cp, cb, OLD_MODE);
                const double* rb = path.GetRMode(*species, lab[b], sl[b], OLD_MODE);
                path.Dr(rc, ra, t);
                for (uint32_t d = 0; d < n_d; ++d) rbar[d] = ra[d] + 0.5 * t[d];
                path.Dr(rb, rbar, delta);
                old_lsp += rho_free_splines[level_i].GetLogRhoFree(delta, n_d);
            }
            {
                float z[4];
                RNG4 wz = st.block(block_base + mid_counter);
                boxmuller(wz.w[0], wz.w[1], z[0], z[1]);
                boxmuller(wz.w[2], wz.w[3], z[2], z[3]);
                mid_counter++;
                for (uint32_t d = 0; d < n_d; ++d) delta[d] = 0. + sigma * (double)z[d];
                path.PutInBox(delta);
                const double* ra = path.GetRMode(*species, lab[a], sl[a], NEW_MODE);
                const double* rc = path.GetRMode(*species, lab[c], sl[c], NEW_MODE);
                path.Dr(rc, ra, t);
                for (uint32_t d = 0; d < n_d; ++d) rbar[d] = ra[d] + 0.5 * t[d];
                double* rb = path.GetRMode(*species, lab[b], sl[b], NEW_MODE);
                for (uint32_t d = 0; d < n_d; ++d) rb[d] = rbar[d] + delta[d];
                new_lsp += rho_free_splines[level_i].GetLogRhoFree(delta, n_d);
            }
        }
    }

    // The beads GetNextBead(0..B) of (p, b0) along the NEW links.
    void Chain(uint32_t p, uint32_t b0, std::vector<uint32_t>& lab, std::vector<uint32_t>& sl) const {
        lab.resize(n_bisect_beads + 1);
        sl.resize(n_bisect_beads + 1);
        lab[0] = p;
        sl[0] = b0;
        for (uint32_t t = 0; t < n_bisect_beads; ++t) {
            lab[t + 1] = path.NextLabel(*species, lab[t], sl[t], NEW_MODE);
            sl[t + 1] = (sl[t] + 1) % species->n_bead;
        }
    }

    double ActionChange(const Particles& parts, int level_i) {
        double old_action = 0., new_action = 0.;
        for (Action* a : action_list) {
            path.mode = OLD_MODE;
            old_action += a->GetAction(bead0, bead1, parts, (uint32_t)level_i);
            path.mode = NEW_MODE;
            new_action += a->GetAction(bead0, bead1, parts, (uint32_t)level_i);
        }
        return new_action - old_action;
    }

    // bisect_class.h:39-124: the segment follows the bead links, and the particle owning the end
    // bead joins the action's particle list when it differs (:61-64).
    bool Attempt() override {
        Stream st{seed, chain, move_index, attempt_counter};
        RNG4 w0 = st.block(0);
        uint32_t p_i = uidx(w0.w[0], species->n_part);
        bead0 = uidx(w0.w[1], species->n_bead);
        bead1 = bead0 + n_bisect_beads;
        std::vector<uint32_t> lab, sl;
        Chain(p_i, bead0, lab, sl);
        affected.clear();
        for (uint32_t i = 0; i <= n_bisect_beads; ++i) affected.push_back({lab[i], sl[i]});
        Particles parts;
        parts.push_back({species->s_i, p_i});
        if (lab[n_bisect_beads] != p_i) parts.push_back({species->s_i, lab[n_bisect_beads]});

        double prev_action_change = 0.;
        uint32_t mid_counter = 0;
        for (int level_i = (int)n_level - 1; level_i >= 0; --level_i) {
            double old_lsp = 0., new_lsp = 0.;
            SampleLevel(st, mid_counter, 1u, level_i, lab, sl, lab[n_bisect_beads], sl[n_bisect_beads], old_lsp, new_lsp);
            double log_sample_ratio = -new_lsp + old_lsp;
            double current = ActionChange(parts, level_i);
            double log_accept = log_sample_ratio - current + prev_action_change;
            RNG4 wu = st.block(1u + (n_bisect_beads - 1u) + (n_level - 1u - (uint32_t)level_i));
            if (log_accept < (double)logf_spec(u24(wu.w[0]))) return false;
            prev_action_change = current;
        }
        return true;
    }

    // bisect_class.h:24-36
    void Accept() override {
        size_t K = path.ks.K();
        for (auto& pb : affected) {
            double* r = path.GetRMode(*species, pb.first, pb.second, NEW_MODE);
            double* rc = path.GetRMode(*species, pb.first, pb.second, OLD_MODE);
            std::copy(r, r + path.n_d, rc);
            if (K && !path.lean_rho) {
                cplx* nw = path.BeadRhoK(*species, pb.first, pb.second, NEW_MODE);
                cplx* od = path.BeadRhoK(*species, pb.first, pb.second, OLD_MODE);
                std::copy(nw, nw + K, od);
            }
        }
        if (K)
            for (uint32_t b = bead0; b < bead1; ++b) {
                uint32_t bb = species->bead_loop(b);
                std::copy(species->rho_k.begin() + (size_t)bb * K, species->rho_k.begin() + (size_t)(bb + 1) * K, species->rho_k_c.begin() + (size_t)bb * K);
            }
        for (Action* a : action_list) a->Accept();
    }

    // bisect_class.h:127-139
    void Reject() override {
        size_t K = path.ks.K();
        for (auto& pb : affected) {
            double* r = path.GetRMode(*species, pb.first, pb.second, NEW_MODE);
            double* rc = path.GetRMode(*species, pb.first, pb.second, OLD_MODE);
            std::copy(rc, rc + path.n_d, r);
            if (K && !path.lean_rho) {
                cplx* nw = path.BeadRhoK(*species, pb.first, pb.second, NEW_MODE);
                cplx* od = path.BeadRhoK(*species, pb.first, pb.second, OLD_MODE);
                std::copy(od, od + K, nw);
            }
        }
        if (K)
            for (uint32_t b = bead0; b < bead1; ++b) {
                uint32_t bb = species->bead_loop(b);
                std::copy(species->rho_k_c.begin() + (size_t)bb * K, species->rho_k_c.begin() + (size_t)(bb + 1) * K, species->rho_k.begin() + (size_t)bb * K);
            }
        for (Action* a : action_list) a->Reject();
    }
};

// ---------------------------------------------------------------------------------------------
// Permuting bisection (perm_bisect_class.h:7-133; perm_bisect_iterative_class.h:7-231 builds the
// cycle particle by particle, perm_bisect_table_class.h:7-240 samples a table of every cycle of
// n_perm_part particles). Random numbers of attempt a of move m come from Philox blocks
// (a, m, block) as for the bisection, laid out by the species' particle count N and B = 2^n_level:
//   block 0                  word 0: first slice; word 1: first particle (iterative); words 2, 3:
//                            the table's selection uniform (53 bits)
//   block 1 + j, j < N       step j of the iterative cycle: words 0, 1 the continuation uniform,
//                            words 2, 3 the choice uniform
//   block 1 + N + c          midpoint c, in the order level, cycle path, position along the path
//   block 1 + N + N(B-1) + l the level test of level n_level - 1 - l (word 0, as the bisection)
//   block 1 + N + N(B-1) + n_level   the table's final test (words 0, 1)
// Departures: the table variant adds the particles owning the end beads to the action's particle
// list when the segment passes the ring closure, as the iterative variant does (:141-146 there;
// the table omits it, which leaves the moved beads beyond the closure out of the label-indexed
// actions and of the density update); the cycle table enumerates permutations and particle subsets
// in lexicographic order (GenPerm / GenCombPermK belong to the absent scaffold library); a cycle
// walk that selects no particle in N steps (only possible by rounding of the running sum) ends
// the attempt as an unselected cycle; a selection uniform at the table's total picks the last cycle.
static double u53(uint32_t a, uint32_t b) { return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0); }

struct PermBisect : Bisect {
    bool table;
    double epsilon, log_epsilon;
    uint32_t n_perm_part = 0, n_perm_type = 0, n_perm_part_in = 0;
    std::vector<uint64_t> perm_attempt, perm_accept;
    std::vector<double> t;  // [N][N]
    struct Cycle {
        double weight = 0., contribution = 0.;
        uint32_t type = 0;
        std::vector<uint32_t> part, perm, i_perm;
    };
    std::vector<Cycle> all_cycles;
    Cycle cyc;
    uint32_t s0 = 0;  // slice of the bead before the permuted link

    PermBisect(Path& p, std::vector<std::unique_ptr<Action>>& actions, const Input& in, uint32_t idx, uint32_t sd, uint32_t ch, bool tbl)
        : Bisect(p, actions, in, idx, sd, ch), table(tbl) {
        epsilon = in.GetAttribute<double>("epsilon", 1.e-100);
        log_epsilon = std::log(epsilon);
        const uint32_t N = species->n_part;
        t.assign((size_t)N * N, 0.);
        perm_attempt.assign(N, 0);
        perm_accept.assign(N, 0);
        if (table) {
            n_perm_part_in = in.GetAttribute<uint32_t>("n_perm_part");
            BuildCycles();
        } else
            n_perm_type = N;
    }

    // perm_bisect_table_class.h:54-102
    void BuildCycles() {
        const uint32_t k = n_perm_part_in, N = species->n_part;
        if (k < 1 || k > N) throw InputError("n_perm_part must be between 1 and the particle count");
        std::vector<std::vector<uint32_t>> perms, combs;
        std::vector<uint32_t> a(k);
        for (uint32_t i = 0; i < k; ++i) a[i] = i;
        do perms.push_back(a);
        while (std::next_permutation(a.begin(), a.end()));
        n_perm_type = (uint32_t)perms.size();
        std::vector<uint32_t> c(k);
        for (uint32_t i = 0; i < k; ++i) c[i] = i;
        while (true) {
            combs.push_back(c);
            int i = (int)k - 1;
            while (i >= 0 && c[i] == N - k + (uint32_t)i) --i;
            if (i < 0) break;
            c[i]++;
            for (uint32_t j = (uint32_t)i + 1; j < k; ++j) c[j] = c[j - 1] + 1;
        }
        for (uint32_t ty = 0; ty < perms.size(); ++ty)
            for (auto& cb : combs) {
                Cycle cy;
                cy.type = ty;
                cy.part = cb;
                cy.perm = perms[ty];
                cy.i_perm.resize(k);
                for (uint32_t j = 0; j < k; ++j) cy.i_perm[cy.perm[j]] = j;
                all_cycles.push_back(cy);
            }
    }

    // UpdatePermTable (perm_bisect_iterative_class.h:10-29, perm_bisect_table_class.h:31-51): the
    // free-particle weight from the start bead of i to the end bead (B links on) of j.
    void UpdateTable() {
        const uint32_t N = species->n_part;
        std::vector<uint32_t> ep(N), eb(N);
        for (uint32_t j = 0; j < N; ++j) ep[j] = path.Walk(*species, j, bead0, n_bisect_beads, NEW_MODE, eb[j]);
        const double i4 = i_4_lambda_tau / n_bisect_beads;
        for (uint32_t i = 0; i < N; ++i) {
            double dii = 0., dr[3];
            path.Dr(path.GetRMode(*species, i, bead0, NEW_MODE), path.GetRMode(*species, ep[i], eb[i], NEW_MODE), dr);
            for (uint32_t d = 0; d < path.n_d; ++d) dii += dr[d] * dr[d];
            for (uint32_t j = 0; j < N; ++j) {
                path.Dr(path.GetRMode(*species, i, bead0, NEW_MODE), path.GetRMode(*species, ep[j], eb[j], NEW_MODE), dr);
                double dij = 0.;
                for (uint32_t d = 0; d < path.n_d; ++d) dij += dr[d] * dr[d];
                const double ex = table ? (-dij + dii) * i4 : (-dij) * i4;
                t[(size_t)i * N + j] = ex > log_epsilon ? std::exp(ex) : 0.;
            }
        }
    }

    // perm_bisect_table_class.h:10-28: returns the total weight; fills `order`/`contrib` with the
    // cycles above epsilon and their running sums.
    double TableTotal(std::vector<uint32_t>* order, std::vector<double>* contrib) {
        UpdateTable();
        const uint32_t N = species->n_part;
        double total = 0.;
        for (uint32_t ci = 0; ci < all_cycles.size(); ++ci) {
            Cycle& c = all_cycles[ci];
            c.weight = 1.;
            for (uint32_t i = 0; i < c.part.size(); ++i) c.weight *= t[(size_t)c.part[i] * N + c.part[c.perm[i]]];
            if (c.weight > epsilon) {
                total += c.weight;
                c.contribution = total;
                if (order) {
                    order->push_back(ci);
                    contrib->push_back(total);
                }
            }
        }
        return total;
    }

    // perm_bisect_iterative_class.h:32-110
    bool SelectIterative(const Stream& st, const RNG4& w0) {
        UpdateTable();
        const uint32_t N = species->n_part;
        std::vector<double> tc = t;
        const uint32_t p0 = uidx(w0.w[1], N);
        uint32_t p = p0;
        std::vector<uint32_t> ps;
        for (uint32_t step = 0;; ++step) {
            if (step >= N) return false;
            ps.push_back(p);
            const size_t n = ps.size();
            for (size_t i = 0; i < n; ++i) tc[(size_t)p * N + ps[i]] = 0.;
            tc[(size_t)p * N + p0] = t[(size_t)p * N + p0];
            double Qp = 0., Qpc = 0.;
            for (uint32_t i = 0; i < N; ++i) {
                Qp += t[(size_t)p * N + i];
                Qpc += tc[(size_t)p * N + i];
            }
            const RNG4 w = st.block(1u + step);
            if (Qpc / Qp < u53(w.w[0], w.w[1])) return false;
            const double x = u53(w.w[2], w.w[3]);
            double tQ = 0.;
            for (uint32_t i = 0; i < N; ++i) {
                tQ += tc[(size_t)p * N + i] / Qpc;
                if (tQ > x) {
                    p = i;
                    break;
                }
            }
            if (p == p0) break;
        }
        const uint32_t n = (uint32_t)ps.size();
        cyc.weight = 1.;
        for (uint32_t i = 0; i + 1 < n; ++i) cyc.weight *= t[(size_t)ps[i] * N + ps[i + 1]] / t[(size_t)ps[i] * N + ps[i]];
        cyc.weight *= t[(size_t)ps[n - 1] * N + ps[0]] / t[(size_t)ps[n - 1] * N + ps[n - 1]];
        cyc.part = ps;
        cyc.type = n - 1;
        cyc.perm.resize(n);
        cyc.i_perm.resize(n);
        for (uint32_t i = 0; i < n; ++i) {
            cyc.perm[i] = (i + 1) % n;
            cyc.i_perm[i] = (i + n - 1) % n;
        }
        return true;
    }

    bool Attempt() override {
        Stream st{seed, chain, move_index, attempt_counter};
        const RNG4 w0 = st.block(0);
        const uint32_t N = species->n_part, M = species->n_bead, B = n_bisect_beads;
        bead0 = uidx(w0.w[0], M);
        bead1 = bead0 + B;
        const bool roll_over = bead1 > M - 1;
        n_perm_part = 0;
        affected.clear();
        double perm_tot_0 = 0.;
        if (table) {
            std::vector<uint32_t> order;
            std::vector<double> contrib;
            perm_tot_0 = TableTotal(&order, &contrib);
            const double x = u53(w0.w[2], w0.w[3]) * perm_tot_0;
            size_t k = 0;
            if (!(x < contrib[0])) {  // SelectCycle, perm_bisect_table_class.h:105-119
                size_t hi = contrib.size(), lo = 0;
                while (hi - lo > 1) {
                    const size_t mid = (hi + lo) >> 1;
                    if (x < contrib[mid]) hi = mid;
                    else lo = mid;
                }
                k = std::min(hi, contrib.size() - 1);
            }
            cyc = all_cycles[order[k]];
        } else if (!SelectIterative(st, w0))
            return false;
        const uint32_t n = (uint32_t)cyc.part.size();
        n_perm_part = n;

        std::vector<std::vector<uint32_t>> lab(n), sl(n);
        for (uint32_t i = 0; i < n; ++i) Chain(cyc.part[i], bead0, lab[i], sl[i]);
        Particles parts;
        for (uint32_t i = 0; i < n; ++i) parts.push_back({species->s_i, cyc.part[i]});
        if (roll_over) {
            for (uint32_t i = 0; i < n; ++i) parts.push_back({species->s_i, lab[i][B]});
            std::sort(parts.begin(), parts.end());
            parts.erase(std::unique(parts.begin(), parts.end()), parts.end());
        }
        // PermuteBeads (perm_bisect_class.h:32-44): the bead before the end of path i now links to
        // the end bead of path perm(i).
        s0 = sl[0][B - 1];
        std::vector<uint32_t> old_end(n);
        for (uint32_t i = 0; i < n; ++i) old_end[i] = lab[i][B];
        for (uint32_t i = 0; i < n; ++i) species->nxt[(size_t)lab[i][B - 1] * M + s0] = old_end[cyc.perm[i]];
        for (uint32_t i = 0; i < n; ++i) lab[i][B] = old_end[cyc.perm[i]];
        for (uint32_t i = 0; i < n; ++i)
            for (uint32_t k = 1; k < B; ++k) affected.push_back({lab[i][k], sl[i][k]});

        double prev_action_change = -std::log(cyc.weight);
        uint32_t mid_counter = 0;
        const uint32_t base_m = 1u + N, base_u = base_m + N * (B - 1u);
        for (int level_i = (int)n_level - 1; level_i >= 0; --level_i) {
            double old_lsp = 0., new_lsp = 0.;
            for (uint32_t i = 0; i < n; ++i) SampleLevel(st, mid_counter, base_m, level_i, lab[i], sl[i], old_end[i], sl[i][B], old_lsp, new_lsp);
            const double current = ActionChange(parts, level_i);
            const double log_accept = -new_lsp + old_lsp - current + prev_action_change;
            const RNG4 wu = st.block(base_u + (n_level - 1u - (uint32_t)level_i));
            if (log_accept < (double)logf_spec(u24(wu.w[0]))) return false;
            prev_action_change = current;
        }
        if (table && n < N) {  // perm_bisect_table_class.h:216-225
            path.mode = NEW_MODE;
            const double perm_tot_1 = TableTotal(nullptr, nullptr);
            const RNG4 wf = st.block(base_u + n_level);
            if (perm_tot_0 / perm_tot_1 < u53(wf.w[0], wf.w[1])) return false;
        }
        return true;
    }

    // AssignParticleLabels (perm_bisect_class.h:47-56): beads after slice s0 take the label of the
    // path that reaches them from slice s0; their positions, densities and links move with them.
    void AssignParticleLabels() {
        const uint32_t N = species->n_part, M = species->n_bead, nd = path.n_d;
        const size_t K = path.ks.K();
        std::vector<uint32_t> src((size_t)N * M);
        for (uint32_t p = 0; p < N; ++p) {
            uint32_t q = p;
            for (uint32_t b = s0; b < M; ++b) {
                src[(size_t)p * M + b] = q;
                if (b + 1 < M) q = path.NextLabel(*species, q, b, NEW_MODE);
            }
        }
        const std::vector<double> r0 = path.r, rc0 = path.r_c;
        const std::vector<cplx> k0 = species->bead_rho_k, kc0 = species->bead_rho_k_c;
        const std::vector<uint32_t> n0 = species->nxt, nc0 = species->nxt_c;
        for (uint32_t p = 0; p < N; ++p) {
            for (uint32_t b = s0 + 1; b < M; ++b) {
                const uint32_t q = src[(size_t)p * M + b];
                std::copy(r0.begin() + path.Idx(*species, q, b), r0.begin() + path.Idx(*species, q, b) + nd, path.r.begin() + path.Idx(*species, p, b));
                std::copy(rc0.begin() + path.Idx(*species, q, b), rc0.begin() + path.Idx(*species, q, b) + nd, path.r_c.begin() + path.Idx(*species, p, b));
                if (K && !path.lean_rho) {
                    std::copy(k0.begin() + ((size_t)q * M + b) * K, k0.begin() + ((size_t)q * M + b + 1) * K, species->bead_rho_k.begin() + ((size_t)p * M + b) * K);
                    std::copy(kc0.begin() + ((size_t)q * M + b) * K, kc0.begin() + ((size_t)q * M + b + 1) * K, species->bead_rho_k_c.begin() + ((size_t)p * M + b) * K);
                }
            }
            for (uint32_t b = s0; b + 1 < M; ++b) species->nxt[(size_t)p * M + b] = species->nxt_c[(size_t)p * M + b] = p;
            const uint32_t q = src[(size_t)p * M + M - 1];
            species->nxt[(size_t)p * M + M - 1] = n0[(size_t)q * M + M - 1];
            species->nxt_c[(size_t)p * M + M - 1] = nc0[(size_t)q * M + M - 1];
        }
    }

    // perm_bisect_class.h:59-73 (the stores of Bisect::Accept act on the moved beads before their
    // relabelling, which carries both copies along)
    void Accept() override {
        const uint32_t M = species->n_bead;
        for (uint32_t p = 0; p < species->n_part; ++p) species->nxt_c[(size_t)p * M + s0] = species->nxt[(size_t)p * M + s0];
        Bisect::Accept();
        if (n_perm_part > 1) AssignParticleLabels();
        perm_attempt[n_perm_part - 1]++;
        perm_accept[n_perm_part - 1]++;
    }

    // perm_bisect_class.h:75-90
    void Reject() override {
        if (n_perm_part > 0) {
            const uint32_t M = species->n_bead;
            for (uint32_t p = 0; p < species->n_part; ++p) species->nxt[(size_t)p * M + s0] = species->nxt_c[(size_t)p * M + s0];
            perm_attempt[n_perm_part - 1]++;
        }
        Bisect::Reject();
    }

    // perm_bisect_class.h:93-97, 119-132 (counters reset at every Write)
    void ResetBlock() override {
        Bisect::ResetBlock();
        std::fill(perm_attempt.begin(), perm_attempt.end(), 0);
        std::fill(perm_accept.begin(), perm_accept.end(), 0);
    }
};

// ---------------------------------------------------------------------------------------------
// Observables (src/events/observables/*).
// Hybrid Monte Carlo of the whole path (the library's <Move type="HMC">): momenta N(0, 1) per
// coordinate of the moving particles in path order, normal j from Philox block 1 + j/4 (two
// Box-Muller pairs per block), leapfrog on H = S(R) + |P|^2/2 with the exact gradient, accepted
// when -dH >= log u with u from block 0, word 0.
struct HMC : Move {
    Path& path;
    std::vector<std::unique_ptr<Action>>& actions;
    uint32_t move_index, seed, chain, n_steps;
    double eps;
    int species = -1;
    std::vector<double> prop;

    HMC(Path& p, std::vector<std::unique_ptr<Action>>& a, const Input& in, uint32_t idx, uint32_t sd, uint32_t ch)
        : path(p), actions(a), move_index(idx), seed(sd), chain(ch) {
        name = in.GetAttribute<std::string>("name");
        type = in.GetAttribute<std::string>("type");
        eps = in.GetAttribute<double>("step_size", 0.01);
        n_steps = in.GetAttribute<uint32_t>("n_steps", 10);
        const std::string sp = in.GetAttribute<std::string>("species", "");
        if (!sp.empty()) species = (int)p.GetSpecies(sp).s_i;
    }

    bool Attempt() override {
        Stream st{seed, chain, move_index, attempt_counter};
        const uint32_t M = path.n_bead, nd = path.n_d;
        std::vector<double> R(path.r_c), P(R.size(), 0.), G(R.size(), 0.);
        uint64_t j = 0;
        for (auto& s : path.species) {
            if (species >= 0 && (uint32_t)species != s.s_i) continue;
            for (uint32_t p = 0; p < s.n_part; ++p)
                for (uint32_t b = 0; b < M; ++b)
                    for (uint32_t d = 0; d < nd; ++d, ++j) {
                        RNG4 w = st.block(1u + (uint32_t)(j >> 2));
                        float z0, z1;
                        if ((j & 3u) < 2) boxmuller(w.w[0], w.w[1], z0, z1);
                        else boxmuller(w.w[2], w.w[3], z0, z1);
                        P[((size_t)(s.offset + p) * M + b) * nd + d] = (double)((j & 1u) ? z1 : z0);
                    }
        }
        auto kin = [&]() {
            double k = 0.;
            for (double x : P) k += 0.5 * x * x;
            return k;
        };
        const double h0 = WholeAction(path, actions, -1, R.data()) + kin();
        WholeGradient(path, actions, -1, R.data(), G.data());
        for (size_t i = 0; i < P.size(); ++i) P[i] -= 0.5 * eps * G[i];
        for (uint32_t s = 0; s < n_steps; ++s) {
            for (size_t i = 0; i < R.size(); ++i) R[i] += eps * P[i];
            WholeGradient(path, actions, -1, R.data(), G.data());
            const double f = s + 1 == n_steps ? 0.5 * eps : eps;
            for (size_t i = 0; i < P.size(); ++i) P[i] -= f * G[i];
        }
        const double h1 = WholeAction(path, actions, -1, R.data()) + kin();
        const double log_accept = -(h1 - h0);
        const double logu = (double)logf_spec(u24(st.block(0).w[0]));
        prop.swap(R);
        return std::isfinite(log_accept) && !(log_accept < logu);
    }
    void Accept() override {
        path.r = prop;
        path.r_c = prop;
        for (auto& s : path.species) path.InitRhoK(s);
    }
    void Reject() override {}
};

struct Observable {
    std::string name, type;
    uint32_t n_measure = 0, skip = 1;
    virtual ~Observable() {}
    virtual void Accumulate() = 0;
    virtual void Reset() = 0;
    // Normalised block values in the order the reference writes them; returns count.
    virtual std::vector<double> Block() = 0;
};

// energy_class.h:7-326 (thermal / virial; potentials optional; no per-sector split)
struct Energy : Observable {
    Path& path;
    std::vector<std::unique_ptr<Action>>& actions;
    bool measure_potential, use_thermal, use_virial, use_adjoint = false;
    uint32_t virial_window_size = 0;
    std::vector<double> energies, potentials;

    Energy(Path& p, std::vector<std::unique_ptr<Action>>& a, const Input& in) : path(p), actions(a) {
        name = in.GetAttribute<std::string>("name");
        type = in.GetAttribute<std::string>("type");
        skip = in.GetAttribute<uint32_t>("skip", 1);
        measure_potential = in.GetAttribute<bool>("measure_potential", false);
        use_virial = in.GetAttribute<bool>("use_virial_estimator", false);
        use_adjoint = in.GetAttribute<bool>("use_adjoint_gradient", false);
        if (use_virial) {
            virial_window_size = in.GetAttribute<uint32_t>("virial_window_size", p.n_bead);
            use_thermal = in.GetAttribute<bool>("use_thermal_estimator", false);
        } else
            use_thermal = in.GetAttribute<bool>("use_thermal_estimator", true);
        energies.assign(actions.size(), 0.);
        potentials.assign(actions.size(), 0.);
    }

    double Thermal(double cof) {
        double tot = 0.;
        for (size_t i = 0; i < actions.size(); ++i) {
            if (actions[i]->is_importance_weight) continue;
            double e = actions[i]->DActionDBeta();
            energies[i] += cof * e;
            tot += e;
        }
        return tot;
    }

    // energy_class.h:36-116
    double Virial(double cof) {
        double ke = 0.;
        for (auto& a : actions)
            if (a->type == "Kinetic") ke += a->VirialEnergy(virial_window_size);
        std::vector<double> G;
        if (use_adjoint) {  // exact gradient of every non-kinetic action, trap and Ewald forces included
            G.assign((size_t)path.n_total * path.n_bead * path.n_d, 0.);
            WholeGradient(path, actions, -2, path.r.data(), G.data());
        }
        for (auto& s : path.species) {
            if (!(s.lambda > 0.)) continue;
            double centroid = 0.;
            if (use_adjoint) {
                for (uint32_t p = 0; p < s.n_part; ++p)
                    for (uint32_t b = 0; b < path.n_bead; ++b) {
                        double dr[3];
                        path.Dr(path.GetR(s, p, b), path.GetR(s, p, 0), dr);
                        const double* g = G.data() + ((size_t)(s.offset + p) * path.n_bead + b) * path.n_d;
                        for (uint32_t d = 0; d < path.n_d; ++d) centroid += g[d] * dr[d];
                    }
            }
            for (uint32_t p = 0; p < s.n_part && !use_adjoint; ++p) {
                Particles parts{{s.s_i, p}};
                for (uint32_t b = 0; b < path.n_bead; ++b) {
                    double dr[3], g[3];
                    path.Dr(path.GetR(s, p, b), path.GetR(s, p, 0), dr);
                    for (size_t i = 0; i < actions.size(); ++i) {
                        if (actions[i]->is_importance_weight || actions[i]->type == "Kinetic") continue;
                        actions[i]->GetActionGradient(b, b + 1, parts, 0, g);
                        for (uint32_t d = 0; d < path.n_d; ++d) centroid += g[d] * dr[d];
                    }
                }
            }
            ke += centroid / (2. * path.tau);
            for (size_t i = 0; i < actions.size(); ++i)
                if (actions[i]->type == "Kinetic")
                    for (uint32_t sp : actions[i]->species_list)
                        if (sp == s.s_i) energies[i] += cof * ke;
        }
        double ie = 0.;
        for (size_t i = 0; i < actions.size(); ++i) {
            if (actions[i]->is_importance_weight || actions[i]->type == "Kinetic") continue;
            double e = actions[i]->DActionDBeta();
            energies[i] += cof * e;
            ie += e;
        }
        return ke + ie;
    }

    void Accumulate() override {
        path.mode = NEW_MODE;
        double cof = path.GetSign();  // sign * importance weight (no importance-weight actions)
        if (use_thermal) Thermal(cof);
        else if (use_virial) Virial(cof);
        if (measure_potential)
            for (size_t i = 0; i < actions.size(); ++i)
                if (!actions[i]->is_importance_weight) potentials[i] += cof * actions[i]->Potential();
        n_measure++;
    }
    void Reset() override {
        n_measure = 0;
        std::fill(energies.begin(), energies.end(), 0.);
        std::fill(potentials.begin(), potentials.end(), 0.);
    }
    // [total, per-action energies..., (v_total, per-action potentials...)] / (M * n_measure)
    std::vector<double> Block() override {
        std::vector<double> out;
        if (n_measure == 0) return out;
        double norm = (double)path.n_bead * n_measure;
        double E = 0.;
        std::vector<double> e(energies.size());
        for (size_t i = 0; i < e.size(); ++i) {
            e[i] = energies[i] / norm;
            E += e[i];
        }
        out.push_back(E);
        out.insert(out.end(), e.begin(), e.end());
        if (measure_potential) {
            double V = 0.;
            std::vector<double> v(potentials.size());
            for (size_t i = 0; i < v.size(); ++i) {
                v[i] = potentials[i] / norm;
                V += v[i];
            }
            out.push_back(V);
            out.insert(out.end(), v.begin(), v.end());
        }
        Reset();
        return out;
    }
};

// pair_correlation_class.h:7-124
struct PairCorrelation : Observable {
    Path& path;
    Species *sa, *sb;
    std::vector<std::pair<uint32_t, uint32_t>> pairs;
    double r_min, r_max, dr, d_ir;
    uint32_t n_r;
    std::vector<double> gr, rs;

    PairCorrelation(Path& p, const Input& in) : path(p) {
        name = in.GetAttribute<std::string>("name");
        type = in.GetAttribute<std::string>("type");
        skip = in.GetAttribute<uint32_t>("skip", 1);
        sa = &p.GetSpecies(in.GetAttribute<std::string>("species_a"));
        sb = &p.GetSpecies(in.GetAttribute<std::string>("species_b"));
        if (sa == sb) {
            for (uint32_t i = 0; i + 1 < sa->n_part; ++i)
                for (uint32_t j = i + 1; j < sb->n_part; ++j) pairs.push_back({i, j});
        } else {
            for (uint32_t i = 0; i < sa->n_part; ++i)
                for (uint32_t j = 0; j < sb->n_part; ++j) pairs.push_back({i, j});
        }
        r_min = in.GetAttribute<double>("r_min", 0.);
        r_max = in.GetAttribute<double>("r_max", p.L / 2.);
        n_r = in.GetAttribute<uint32_t>("n_r", 100);
        if (n_r < 2) throw InputError("n_r must be at least 2");
        dr = (r_max - r_min) / (n_r - 1.);  // observable_class.h:29-38
        d_ir = 1. / dr;
        rs.resize(n_r);
        for (uint32_t i = 0; i < n_r; ++i) rs[i] = r_min + i * dr;
        gr.assign(n_r, 0.);
    }
    // observable_class.h:56-62
    uint32_t ReverseMap(double r) const { return (uint32_t)std::nearbyint((r - r_min) * d_ir - 0.5); }
    void Accumulate() override {
        path.mode = NEW_MODE;
        double cof = path.GetSign();
        double t[3];
        for (uint32_t b = 0; b < path.n_bead; ++b)
            for (auto& pr : pairs) {
                path.Dr(path.GetR(*sa, pr.first, b), path.GetR(*sb, pr.second, b), t);
                double m = 0.;
                for (uint32_t d = 0; d < path.n_d; ++d) m += t[d] * t[d];
                uint32_t i = ReverseMap(std::sqrt(m));
                if (i < n_r) gr[i] = gr[i] + 1. * cof;
            }
        n_measure++;
    }
    void Reset() override {
        n_measure = 0;
        std::fill(gr.begin(), gr.end(), 0.);
    }
    std::vector<double> Block() override {
        std::vector<double> out;
        if (n_measure == 0) return out;
        double norm;
        if (sa == sb) norm = 0.5 * n_measure * sa->n_part * (sb->n_part - 1) * path.n_bead / path.vol;
        else norm = (double)n_measure * sa->n_part * sb->n_part * path.n_bead / path.vol;
        out.resize(n_r);
        for (uint32_t i = 0; i < n_r; ++i) {
            double r1 = rs[i];
            double r2 = (i < n_r - 1) ? rs[i + 1] : (2. * rs[i] - rs[i - 1]);
            double bin_vol;
            if (path.n_d == 3) bin_vol = 4. * M_PI / 3. * (r2 * r2 * r2 - r1 * r1 * r1);
            else if (path.n_d == 2) bin_vol = M_PI * (r2 * r2 - r1 * r1);
            else bin_vol = r2 - r1;
            out[i] = gr[i] / (bin_vol * norm);
        }
        Reset();
        return out;
    }
};

// structure_factor_class.h:7-86
struct StructureFactor : Observable {
    Path& path;
    Species *sa, *sb;
    double k_cut;
    std::vector<double> sk;

    StructureFactor(Path& p, const Input& in) : path(p) {
        name = in.GetAttribute<std::string>("name");
        type = in.GetAttribute<std::string>("type");
        skip = in.GetAttribute<uint32_t>("skip", 1);
        sa = &p.GetSpecies(in.GetAttribute<std::string>("species_a"));
        sb = &p.GetSpecies(in.GetAttribute<std::string>("species_b"));
        if (!p.pbc) throw InputError("StructureFactor needs periodic boundaries");
        k_cut = in.GetAttribute<double>("k_cut", p.ks.cutoff);
        p.ks.Setup(k_cut);
    }
    void Init() { sk.assign(path.ks.K(), 0.); }
    void Accumulate() override {
        path.mode = NEW_MODE;
        const double cof = path.GetSign();
        const auto& ra = path.GetRhoK(*sa);
        const auto& rb = path.GetRhoK(*sb);
        size_t K = path.ks.K();
        for (size_t k = 0; k < K; ++k)
            if (path.ks.mags[k] < k_cut)
                for (uint32_t b = 0; b < path.n_bead; ++b) sk[k] += cof * CMag2(ra[(size_t)b * K + k], rb[(size_t)b * K + k]);
        n_measure++;
    }
    void Reset() override {
        n_measure = 0;
        std::fill(sk.begin(), sk.end(), 0.);
    }
    std::vector<double> Block() override {
        std::vector<double> out;
        if (n_measure == 0) return out;
        double norm = (double)n_measure * path.n_bead * sa->n_part * sb->n_part;
        out.resize(sk.size());
        for (size_t k = 0; k < sk.size(); ++k) out[k] = sk[k] / norm;
        Reset();
        return out;
    }
};

// sign_class.h:7-48: the block mean of the path's sign.
struct SignObs : Observable {
    Path& path;
    double sign = 0.;
    SignObs(Path& p, const Input& in) : path(p) {
        name = in.GetAttribute<std::string>("name");
        type = in.GetAttribute<std::string>("type");
    }
    void Accumulate() override {
        sign += path.GetSign();
        n_measure++;
    }
    void Reset() override {
        n_measure = 0;
        sign = 0.;
    }
    std::vector<double> Block() override {
        std::vector<double> out;
        if (n_measure == 0) return out;
        out.push_back(sign / n_measure);
        Reset();
        return out;
    }
};

// permutation_class.h:7-119: the normalised histogram of cycle lengths, then the (sector, count)
// pairs of the block in increasing sector order. Sectors are the partitions of N into cycle
// lengths, numbered in the order the ascending-composition generation of species_class.h:178-221
// produces them (the reference's guard there skips the generation, leaving the lookup of :172-175
// without entries; the numbering it intends is used).
struct PermutationObs : Observable {
    Path& path;
    Species* species;
    std::vector<double> cycles;
    std::vector<uint32_t> sectors;
    std::vector<std::vector<uint32_t>> partitions;
    PermutationObs(Path& p, const Input& in) : path(p) {
        name = in.GetAttribute<std::string>("name");
        type = in.GetAttribute<std::string>("type");
        species = &p.GetSpecies(in.GetAttribute<std::string>("species"));
        const uint32_t sector_max = in.GetAttribute<uint32_t>("sector_max", 0);
        partitions = Partitions(species->n_part, sector_max);
        cycles.assign(species->n_part, 0.);
    }
    // Accelerated ascending-composition generation of the partitions of n (Kelleher and O'Sullivan).
    static std::vector<std::vector<uint32_t>> Partitions(uint32_t n, uint32_t cap) {
        std::vector<std::vector<uint32_t>> out;
        if (n == 0) return out;
        std::vector<uint32_t> a(n + 1, 0);
        uint32_t k = 1, y = n - 1;
        auto room = [&]() { return cap == 0 || out.size() < cap; };
        while (k != 0 && room()) {
            uint32_t x = a[k - 1] + 1;
            k -= 1;
            while (2 * x <= y) {
                a[k] = x;
                y -= x;
                k += 1;
            }
            const uint32_t l = k + 1;
            while (x <= y && room()) {
                a[k] = x;
                a[l] = y;
                out.emplace_back(a.begin(), a.begin() + k + 2);
                x += 1;
                y -= 1;
            }
            a[k] = x + y;
            y = x + y - 1;
            out.emplace_back(a.begin(), a.begin() + k + 1);
        }
        return out;
    }
    std::vector<uint32_t> CycleLengths() const {
        std::vector<uint32_t> out;
        std::vector<char> seen(species->n_part, 0);
        for (uint32_t p = 0; p < species->n_part; ++p) {
            if (seen[p]) continue;
            uint32_t len = 0, q = p;
            do {
                seen[q] = 1;
                q = path.NextLabel(*species, q, species->n_bead - 1, NEW_MODE);
                ++len;
            } while (q != p);
            out.push_back(len);
        }
        return out;
    }
    void Accumulate() override {
        auto c = CycleLengths();
        for (uint32_t l : c) cycles[l - 1] += 1.;
        std::sort(c.begin(), c.end());
        uint32_t sector = (uint32_t)partitions.size();  // not among the first sector_max partitions
        for (size_t i = 0; i < partitions.size(); ++i)
            if (partitions[i] == c) sector = (uint32_t)i;
        sectors.push_back(sector);
        n_measure++;
    }
    void Reset() override {
        n_measure = 0;
        std::fill(cycles.begin(), cycles.end(), 0.);
        sectors.clear();
    }
    std::vector<double> Block() override {
        std::vector<double> out;
        if (n_measure == 0) return out;
        double n_cycles = 0.;
        for (double c : cycles) n_cycles += c;
        for (double c : cycles) out.push_back(c / n_cycles);
        std::vector<uint32_t> s = sectors;
        std::sort(s.begin(), s.end());
        for (size_t i = 0; i < s.size();) {
            size_t j = i;
            while (j < s.size() && s[j] == s[i]) ++j;
            out.push_back((double)s[i]);
            out.push_back((double)(j - i));
            i = j;
        }
        Reset();
        return out;
    }
};

// ---------------------------------------------------------------------------------------------
// Simulation (src/framework/simulation_class.h:8-46) with the Loop/Write events (loop_class.h).
struct LoopNode {
    int kind = 0;  // 0 loop, 1 move, 2 observable, 3 write
    uint32_t index = 0;
    uint64_t n_steps = 1;
    std::vector<LoopNode> children;
};

struct Simulation {
    std::string base_dir;
    uint32_t seed = 12345, chain = 0;
    std::unique_ptr<Path> path;
    std::vector<std::unique_ptr<Action>> actions;
    std::vector<std::unique_ptr<Move>> moves;
    std::vector<std::unique_ptr<Observable>> observables;
    std::vector<uint64_t> obs_calls;
    LoopNode main_loop;
    std::vector<std::vector<std::vector<double>>> blocks;  // per observable, per block
    // per move, per Write: {n_attempt, n_accept, bisection level (adaptive moves; else -1)}, then the
    // per-cycle-length attempts and accepts of a permuting move (move_class.h:80-94,
    // perm_bisect_class.h:119-132)
    std::vector<std::vector<std::vector<int64_t>>> move_writes;

    Simulation(const Input& in, const std::string& bd, uint32_t chain_id) : base_dir(bd), chain(chain_id) {
        Input rng = in.GetChild("RNG");
        seed = rng.IsNull() ? (uint32_t)time(nullptr) : (uint32_t)rng.GetAttribute<int>("seed", (int)time(nullptr));
        path.reset(new Path(in));
        for (auto& a : in.GetChild("Actions").GetChildList("Action")) {
            std::string t = a.GetAttribute<std::string>("type");
            if (t == "Kinetic") actions.emplace_back(new Kinetic(*path, a));
            else if (t == "HarmonicTrap") actions.emplace_back(new Trap(*path, a));
            else if (t == "BarePairAction") actions.emplace_back(new BarePairAction(*path, a, base_dir));
            else if (t == "IlkkaPairAction") actions.emplace_back(new IlkkaPairAction(*path, a, base_dir));
            else if (t == "DavidPairAction") actions.emplace_back(new DavidPairAction(*path, a, base_dir));
            else throw InputError("unsupported action type '" + t + "'");
        }
        uint32_t mi = 0;
        for (auto& m : in.GetChild("Moves").GetChildList("Move")) {
            std::string t = m.GetAttribute<std::string>("type");
            if (t == "Bisect") moves.emplace_back(new Bisect(*path, actions, m, mi, seed, chain));
            else if (t == "HMC") moves.emplace_back(new HMC(*path, actions, m, mi, seed, chain));
            else if (t == "PermBisectIterative") moves.emplace_back(new PermBisect(*path, actions, m, mi, seed, chain, false));
            else if (t == "PermBisectTable") moves.emplace_back(new PermBisect(*path, actions, m, mi, seed, chain, true));
            else throw InputError("unsupported move type '" + t + "'");
            ++mi;
        }
        for (auto& o : in.GetChild("Observables").GetChildList("Observable")) {
            std::string t = o.GetAttribute<std::string>("type");
            if (t == "Energy") observables.emplace_back(new Energy(*path, actions, o));
            else if (t == "PairCorrelation") observables.emplace_back(new PairCorrelation(*path, o));
            else if (t == "StructureFactor") observables.emplace_back(new StructureFactor(*path, o));
            else if (t == "Sign") observables.emplace_back(new SignObs(*path, o));
            else if (t == "Permutation") observables.emplace_back(new PermutationObs(*path, o));
            else if (t == "Time" || t == "PathDump") continue;  // bookkeeping only
            else throw InputError("unsupported observable type '" + t + "'");
        }
        obs_calls.assign(observables.size(), 0);
        blocks.resize(observables.size());
        // The reference sizes each long-range table at construction (bare_pair_action_class.h:79) and
        // would read past it if a later element grew the k-vector set; refuse that input instead.
        for (auto& a : actions)
            if (a->type == "BarePairAction") {
                auto* b = static_cast<BarePairAction*>(a.get());
                if (b->use_long_range && b->v_long_k.size() != path->ks.K())
                    throw InputError("k_cut of action '" + b->name + "' is below a later k_cut; order the largest first");
            } else if (a->type == "DavidPairAction") {
                auto* b = static_cast<DavidPairAction*>(a.get());
                if (b->use_long_range && b->u_long_k.size() != path->ks.K())
                    throw InputError("k_cut of action '" + b->name + "' is below a later k_cut; order the largest first");
            } else if (a->type == "IlkkaPairAction") {
                auto* b = static_cast<IlkkaPairAction*>(a.get());
                if (b->use_long_range && b->u_long_k.size() != path->ks.K())
                    throw InputError("k_cut of action '" + b->name + "' is below a later k_cut; order the largest first");
            }
        for (auto& o : observables)
            if (o->type == "StructureFactor") static_cast<StructureFactor*>(o.get())->Init();
        for (auto& s : path->species) path->InitRhoK(s);
        Input alg = in.GetChild("Algorithm");
        main_loop.kind = 0;
        main_loop.n_steps = 1;
        ReadLoop(alg, main_loop);
    }

    void ReadLoop(const Input& in, LoopNode& node) {
        for (auto& c : in.GetChildList()) {
            const std::string& t = c.GetName();
            LoopNode ch;
            if (t == "Move" || t == "Observable") {
                std::string nm = c.GetAttribute<std::string>("name");
                bool found = false;
                if (t == "Move") {
                    for (size_t i = 0; i < moves.size(); ++i)
                        if (moves[i]->name == nm) {
                            ch.kind = 1;
                            ch.index = (uint32_t)i;
                            found = true;
                        }
                } else {
                    for (size_t i = 0; i < observables.size(); ++i)
                        if (observables[i]->name == nm) {
                            ch.kind = 2;
                            ch.index = (uint32_t)i;
                            found = true;
                        }
                }
                if (!found) continue;  // loop_class.h:40-44 warns and skips
            } else if (t == "Write") {
                ch.kind = 3;
            } else if (t == "Loop") {
                ch.kind = 0;
                ch.n_steps = (uint64_t)c.GetAttribute<int>("n_step");
                ReadLoop(c, ch);
            } else
                continue;
            node.children.push_back(ch);
        }
    }

    void Write() {
        for (size_t i = 0; i < observables.size(); ++i) {
            auto v = observables[i]->Block();
            if (!v.empty()) blocks[i].push_back(v);
        }
        move_writes.resize(moves.size());
        for (size_t i = 0; i < moves.size(); ++i) {
            Move* m = moves[i].get();
            std::vector<int64_t> row{(int64_t)m->n_attempt, (int64_t)m->n_accept, -1};
            if (auto* b = dynamic_cast<Bisect*>(m))
                if (b->adaptive) row[2] = b->n_level;
            if (auto* pb = dynamic_cast<PermBisect*>(m)) {
                row.insert(row.end(), pb->perm_attempt.begin(), pb->perm_attempt.end());
                row.insert(row.end(), pb->perm_accept.begin(), pb->perm_accept.end());
            }
            move_writes[i].push_back(row);
            m->ResetBlock();
        }
    }

    void RunNode(const LoopNode& n) {
        for (uint64_t s = 0; s < n.n_steps; ++s)
            for (auto& c : n.children) {
                if (c.kind == 0) RunNode(c);
                else if (c.kind == 1) moves[c.index]->DoEvent();
                else if (c.kind == 2)
                    observables[c.index]->Accumulate();  // observable_class.h:93-101 ignores `skip`
                else
                    Write();
            }
    }
};

}  // namespace orc

// =============================================================================================
// C interface used by the tests (ctypes) and by the bench's CPU-baseline leg.
namespace {
thread_local std::string g_err;
int fail(const std::exception& e) {
    g_err = e.what();
    return -1;
}
orc::Simulation* S(void* h) { return static_cast<orc::Simulation*>(h); }
orc::Particles parts_of(const uint32_t* sp, const uint32_t* p, uint32_t n) {
    orc::Particles out;
    for (uint32_t i = 0; i < n; ++i) out.push_back({sp[i], p[i]});
    return out;
}
}  // namespace

extern "C" {

const char* oracle_last_error() { return g_err.c_str(); }

int oracle_create(const char* xml_text, const char* base_dir, uint32_t chain, void** out) {
    try {
        pimc::Input in = pimc::Input::FromString(xml_text);
        *out = new orc::Simulation(in, base_dir ? base_dir : "", chain);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

void oracle_destroy(void* h) { delete S(h); }

// [n_d, n_bead, n_species, n_total, K, n_actions, n_moves, n_observables]
int oracle_info(void* h, uint32_t* out) {
    auto* s = S(h);
    out[0] = s->path->n_d;
    out[1] = s->path->n_bead;
    out[2] = (uint32_t)s->path->species.size();
    out[3] = s->path->n_total;
    out[4] = (uint32_t)s->path->ks.K();
    out[5] = (uint32_t)s->actions.size();
    out[6] = (uint32_t)s->moves.size();
    out[7] = (uint32_t)s->observables.size();
    return 0;
}

int oracle_seed(void* h, uint32_t seed) {
    auto* s = S(h);
    s->seed = seed;
    for (auto& m : s->moves) static_cast<orc::Bisect*>(m.get())->seed = seed;
    return 0;
}

// which: 0 = old copy, 1 = new copy, 2 = both (then charge densities are re-initialised).
int oracle_set_path(void* h, int which, const double* pos) {
    auto* s = S(h);
    size_t n = s->path->r.size();
    if (which == 1 || which == 2) std::copy(pos, pos + n, s->path->r.begin());
    if (which == 0 || which == 2) std::copy(pos, pos + n, s->path->r_c.begin());
    if (which == 2)
        for (auto& sp : s->path->species) sp.need_update_rho_k = true;
    if (which == 2)
        for (auto& sp : s->path->species) s->path->InitRhoK(sp);
    return 0;
}

int oracle_get_path(void* h, int which, double* pos) {
    auto* s = S(h);
    const auto& v = which == 0 ? s->path->r_c : s->path->r;
    std::copy(v.begin(), v.end(), pos);
    return 0;
}

int oracle_kvecs(void* h, double* out) {
    auto* s = S(h);
    for (size_t k = 0; k < s->path->ks.K(); ++k)
        for (uint32_t d = 0; d < s->path->n_d; ++d) out[k * s->path->n_d + d] = s->path->ks.vecs[k][d];
    return 0;
}

int oracle_get_rho_k(void* h, uint32_t species, int which, double* out) {
    auto* s = S(h);
    const auto& sp = s->path->species.at(species);
    const auto& v = which == 0 ? sp.rho_k_c : sp.rho_k;
    for (size_t i = 0; i < v.size(); ++i) {
        out[2 * i] = v[i].real();
        out[2 * i + 1] = v[i].imag();
    }
    return 0;
}

int oracle_get_action(void* h, uint32_t a, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n, uint32_t level,
                      int mode, double* out) {
    try {
        auto* s = S(h);
        s->path->mode = mode ? orc::NEW_MODE : orc::OLD_MODE;
        *out = s->actions.at(a)->GetAction(b0, b1, parts_of(sp, p, n), level);
        s->path->mode = orc::NEW_MODE;
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int oracle_get_action_gradient(void* h, uint32_t a, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n,
                               uint32_t level, int mode, double* out) {
    try {
        auto* s = S(h);
        s->path->mode = mode ? orc::NEW_MODE : orc::OLD_MODE;
        s->actions.at(a)->GetActionGradient(b0, b1, parts_of(sp, p, n), level, out);
        s->path->mode = orc::NEW_MODE;
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// Mark every species' charge density as needing an update (the state after Accept/Reject).
int oracle_reset_rho_k_latch(void* h) {
    for (auto& sp : S(h)->path->species) sp.need_update_rho_k = true;
    return 0;
}

int oracle_dactiondbeta(void* h, uint32_t a, double* out) {
    auto* s = S(h);
    s->path->mode = orc::NEW_MODE;
    *out = s->actions.at(a)->DActionDBeta();
    return 0;
}

int oracle_potential(void* h, uint32_t a, double* out) {
    auto* s = S(h);
    s->path->mode = orc::NEW_MODE;
    *out = s->actions.at(a)->Potential();
    return 0;
}

int oracle_virial_energy(void* h, uint32_t a, double window, double* out) {
    auto* s = S(h);
    s->path->mode = orc::NEW_MODE;
    *out = s->actions.at(a)->VirialEnergy(window);
    return 0;
}

// Whole-ring action (action >= 0, or -1 for every action) and its exact gradient [n_total][M][n_d]
// on the stored (mode 0) or working (mode 1) copy.
int oracle_total_action(void* h, int a, int mode, double* out) {
    try {
        auto* s = S(h);
        *out = orc::WholeAction(*s->path, s->actions, a, mode ? s->path->r.data() : s->path->r_c.data());
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int oracle_action_gradient_path(void* h, int a, int mode, double* out) {
    try {
        auto* s = S(h);
        orc::WholeGradient(*s->path, s->actions, a, mode ? s->path->r.data() : s->path->r_c.data(), out);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int oracle_move_attempts(void* h, uint32_t m, uint64_t n) {
    auto* s = S(h);
    for (uint64_t i = 0; i < n; ++i) s->moves.at(m)->DoEvent();
    return 0;
}

int oracle_move_stats(void* h, uint32_t m, uint64_t* out) {
    // {total attempts, attempts in the current block, accepts in the current block}
    auto* mv = S(h)->moves.at(m).get();
    out[0] = mv->attempt_counter;
    out[1] = mv->n_attempt;
    out[2] = mv->n_accept;
    return 0;
}

// Per cycle length n: attempts and accepts of a permuting move in the current block
// (perm_bisect_class.h:25-26); out[2 N].
int oracle_perm_stats(void* h, uint32_t m, uint64_t* out) {
    try {
        auto* mv = dynamic_cast<orc::PermBisect*>(S(h)->moves.at(m).get());
        if (!mv) throw std::invalid_argument("not a permuting move");
        const size_t N = mv->perm_attempt.size();
        for (size_t i = 0; i < N; ++i) {
            out[i] = mv->perm_attempt[i];
            out[N + i] = mv->perm_accept[i];
        }
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

// The path permutation of a species: out[p] = particle whose slice-0 bead follows (p, M - 1).
int oracle_get_perm(void* h, uint32_t sp, uint32_t* out) {
    try {
        auto& path = *S(h)->path;
        auto pi = path.Closure(path.species.at(sp));
        std::copy(pi.begin(), pi.end(), out);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int oracle_set_perm(void* h, uint32_t sp, const uint32_t* pi) {
    try {
        auto& path = *S(h)->path;
        auto& s = path.species.at(sp);
        std::vector<char> seen(s.n_part, 0);
        for (uint32_t p = 0; p < s.n_part; ++p) {
            if (pi[p] >= s.n_part || seen[pi[p]]) throw std::invalid_argument("not a permutation");
            seen[pi[p]] = 1;
        }
        for (uint32_t p = 0; p < s.n_part; ++p) s.nxt[(size_t)p * s.n_bead + s.n_bead - 1] = s.nxt_c[(size_t)p * s.n_bead + s.n_bead - 1] = pi[p];
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int oracle_obs_accumulate(void* h, uint32_t o) {
    S(h)->observables.at(o)->Accumulate();
    return 0;
}

// Normalised block of observable o (the values its Write() would append); resets it.
int oracle_obs_block(void* h, uint32_t o, double* out, uint64_t cap, uint64_t* n) {
    auto v = S(h)->observables.at(o)->Block();
    *n = v.size();
    for (size_t i = 0; i < v.size() && i < cap; ++i) out[i] = v[i];
    return 0;
}

// Runs the input's Algorithm loop; block values are collected per observable.
int oracle_run(void* h) {
    try {
        auto* s = S(h);
        s->RunNode(s->main_loop);
        return 0;
    } catch (const std::exception& e) {
        return fail(e);
    }
}

int oracle_n_blocks(void* h, uint32_t o, uint64_t* n) {
    if (o >= S(h)->blocks.size()) return -1;
    *n = S(h)->blocks[o].size();
    return 0;
}

// Rows recorded at each Write of the last run for move m: {n_attempt, n_accept, level or -1}, and
// for a permuting move its per-cycle-length attempts then accepts (N each); row-major into out.
int oracle_move_writes(void* h, uint32_t m, int64_t* out, uint64_t cap, uint64_t* n_rows, uint64_t* row_len) {
    auto* s = S(h);
    if (m >= s->moves.size()) return -1;
    *n_rows = m < s->move_writes.size() ? s->move_writes[m].size() : 0;
    *row_len = *n_rows ? s->move_writes[m][0].size() : 0;
    uint64_t k = 0;
    for (uint64_t r = 0; r < *n_rows; ++r)
        for (int64_t v : s->move_writes[m][r])
            if (k < cap) out[k++] = v;
    return 0;
}

int oracle_get_block(void* h, uint32_t o, uint64_t blk, double* out, uint64_t cap, uint64_t* n) {
    if (o >= S(h)->blocks.size() || blk >= S(h)->blocks[o].size()) return -1;
    const auto& v = S(h)->blocks[o][blk];
    *n = v.size();
    for (size_t i = 0; i < v.size() && i < cap; ++i) out[i] = v[i];
    return 0;
}

// Draws of one bisection attempt: p, bead0, the 3 normals of each of the (n_bisect - 1) beads and
// the acceptance logarithm of each level, as the move consumes them.
int oracle_bisect_draws(uint32_t seed, uint32_t chain, uint32_t move, uint64_t attempt, uint32_t n_part, uint32_t n_bead, uint32_t n_level,
                        uint32_t* pb, float* z, float* logu) {
    orc::Stream st{seed, chain, move, attempt};
    orc::RNG4 w0 = st.block(0);
    pb[0] = orc::uidx(w0.w[0], n_part);
    pb[1] = orc::uidx(w0.w[1], n_bead);
    const uint32_t B = 1u << n_level;
    for (uint32_t i = 0; i + 1 < B; ++i) {
        orc::RNG4 w = st.block(1u + i);
        float z3;
        orc::boxmuller(w.w[0], w.w[1], z[3 * i], z[3 * i + 1]);
        orc::boxmuller(w.w[2], w.w[3], z[3 * i + 2], z3);
    }
    for (uint32_t li = 0; li < n_level; ++li) logu[li] = orc::logf_spec(orc::u24(st.block(1u + (B - 1u) + li).w[0]));
    return 0;
}

// Draws of one permuting-bisection attempt (the layout above PermBisect), in the order the
// reference's PermBisectIterative / PermBisectTable consume them: idx = {first bead, the iterative
// cycle's first particle}; sel[2 N] = each cycle step's continuation and choice uniforms, then
// sel[2 N] = the table's selection uniform; z = the 3 normals of each of the N (B - 1) midpoints in
// sampling order; logu = the level tests' logarithms, top level first; fin = the table's final
// uniform.
int oracle_perm_draws(uint32_t seed, uint32_t chain, uint32_t move, uint64_t attempt, uint32_t n_part, uint32_t n_bead, uint32_t n_level,
                      uint32_t* idx, double* sel, float* z, float* logu, double* fin) {
    orc::Stream st{seed, chain, move, attempt};
    const orc::RNG4 w0 = st.block(0);
    const uint32_t N = n_part, B = 1u << n_level;
    idx[0] = orc::uidx(w0.w[0], n_bead);
    idx[1] = orc::uidx(w0.w[1], N);
    for (uint32_t j = 0; j < N; ++j) {
        const orc::RNG4 w = st.block(1u + j);
        sel[2 * j] = orc::u53(w.w[0], w.w[1]);
        sel[2 * j + 1] = orc::u53(w.w[2], w.w[3]);
    }
    sel[2 * N] = orc::u53(w0.w[2], w0.w[3]);
    const uint32_t base_m = 1u + N, base_u = base_m + N * (B - 1u);
    for (uint32_t c = 0; c < N * (B - 1u); ++c) {
        const orc::RNG4 w = st.block(base_m + c);
        float z3;
        orc::boxmuller(w.w[0], w.w[1], z[3 * c], z[3 * c + 1]);
        orc::boxmuller(w.w[2], w.w[3], z[3 * c + 2], z3);
    }
    for (uint32_t l = 0; l < n_level; ++l) logu[l] = orc::logf_spec(orc::u24(st.block(base_u + l).w[0]));
    const orc::RNG4 wf = st.block(base_u + n_level);
    fin[0] = orc::u53(wf.w[0], wf.w[1]);
    return 0;
}

// Lean densities for every sim created afterwards (see g_lean_densities).
int oracle_set_lean_densities(int on) {
    orc::g_lean_densities = on != 0;
    return 0;
}

int oracle_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
    orc::RNG4 r = orc::philox(c, key[0], key[1]);
    for (int i = 0; i < 4; ++i) out[i] = r.w[i];
    return 0;
}

}  // extern "C"
