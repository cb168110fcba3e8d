// XML-driven construction of a Context: path, k-space, tables, actions, moves, observables and the
// algorithm loop. Follows the construction order of the reference's Simulation
// (src/framework/simulation_class.h:16-39) and Path (src/data_structures/path_class.h:25-69).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <ctime>

#include "context.h"
#include "table_io.h"

namespace pimc {

void CudaCheck(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw PimcError(kErrCuda, std::string(what) + ": " + cudaGetErrorString(e));
}

DeviceBuffer::DeviceBuffer(size_t n) : bytes(n) {
    if (n == 0) n = 16;
    CudaCheck(cudaMalloc(&ptr, n), "cudaMalloc");
    // cudaMemset runs on the legacy default stream and returns before it completes; the contexts'
    // streams are non-blocking, so without this wait a copy enqueued on a context stream right after
    // the allocation could land first and then be zeroed.
    CudaCheck(cudaMemset(ptr, 0, n), "cudaMemset");
    CudaCheck(cudaStreamSynchronize(cudaStreamLegacy), "cudaMemset completion");
}

DeviceBuffer::~DeviceBuffer() {
    if (ptr) cudaFree(ptr);
}

template <class T>
T* Context::Upload(const std::vector<T>& v) {
    keep_.emplace_back(new DeviceBuffer(v.size() * sizeof(T)));
    if (!v.empty()) CudaCheck(cudaMemcpy(keep_.back()->ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
    return keep_.back()->as<T>();
}

// Natural cubic interpolating spline (second derivatives zero at both ends), the function that
// einspline's {NATURAL, NATURAL} B-spline interpolants represent. Solved by the tridiagonal
// (Thomas) recurrence and stored as one polynomial per interval.
CubicTable Context::BuildCubic(const std::vector<double>& x, const std::vector<double>& y, bool uniform) {
    const size_t n = x.size();
    if (n < 2 || y.size() != n) throw PimcError(kErrInput, "spline needs at least two matching knots");
    for (size_t i = 1; i < n; ++i)
        if (!(x[i] > x[i - 1])) throw PimcError(kErrInput, "spline knots must increase");
    std::vector<double> m(n, 0.);
    if (n >= 3) {
        std::vector<double> cp(n, 0.), dp(n, 0.);
        for (size_t i = 1; i + 1 < n; ++i) {
            const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
            double diag = 2. * (h0 + h1);
            double rhs = 6. * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
            if (i > 1) {
                diag -= h0 * cp[i - 1];
                rhs -= h0 * dp[i - 1];
            }
            cp[i] = h1 / diag;
            dp[i] = rhs / diag;
        }
        m[n - 2] = dp[n - 2];
        for (size_t i = n - 2; i-- > 1;) m[i] = dp[i] - cp[i] * m[i + 1];
    }
    std::vector<Cubic4> c(n - 1);
    for (size_t i = 0; i + 1 < n; ++i) {
        const double h = x[i + 1] - x[i];
        c[i].c0 = y[i];
        c[i].c1 = (y[i + 1] - y[i]) / h - h * (2. * m[i] + m[i + 1]) / 6.;
        c[i].c2 = 0.5 * m[i];
        c[i].c3 = (m[i + 1] - m[i]) / (6. * h);
    }
    CubicTable t;
    t.n = (int32_t)n;
    t.x0 = x.front();
    t.x1 = x.back();
    t.uniform = uniform ? 1 : 0;
    t.x = Upload(x);
    t.c = Upload(c);
    if (uniform) {
        t.inv_dx = (double)(n - 1) / (x.back() - x.front());
    } else {
        // Buckets of equal width over [x0, x1]; each stores the interval holding its left edge.
        const int nb = (int)std::min<size_t>(4 * n, 1u << 20);
        t.n_bucket = nb;
        t.inv_dx = nb / (x.back() - x.front());
        std::vector<int32_t> bk(nb);
        size_t i = 0;
        for (int j = 0; j < nb; ++j) {
            const double xl = x.front() + j / t.inv_dx;
            while (i + 2 < n && x[i + 1] <= xl) ++i;
            bk[j] = (int32_t)i;
        }
        t.bucket = Upload(bk);
        host_cubics.push_back({t.c, HostCubic{x, c, bk}});
        return t;
    }
    host_cubics.push_back({t.c, HostCubic{x, c, {}}});
    return t;
}

// Second derivatives of the natural cubic spline through (x_i, y_i) (zero at both ends).
static std::vector<double> NaturalSecond(const std::vector<double>& x, const std::vector<double>& y) {
    const size_t n = x.size();
    std::vector<double> m(n, 0.);
    if (n < 3) return m;
    std::vector<double> cp(n, 0.), dp(n, 0.);
    for (size_t i = 1; i + 1 < n; ++i) {
        const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
        double diag = 2. * (h0 + h1);
        double rhs = 6. * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
        if (i > 1) {
            diag -= h0 * cp[i - 1];
            rhs -= h0 * dp[i - 1];
        }
        cp[i] = h1 / diag;
        dp[i] = rhs / diag;
    }
    m[n - 2] = dp[n - 2];
    for (size_t i = n - 2; i-- > 1;) m[i] = dp[i] - cp[i] * m[i + 1];
    return m;
}

// First derivatives at the knots of the natural cubic spline through (x_i, y_i).
static std::vector<double> NaturalSlopes(const std::vector<double>& x, const std::vector<double>& y) {
    const size_t n = x.size();
    const std::vector<double> m = NaturalSecond(x, y);
    std::vector<double> d(n);
    for (size_t i = 0; i + 1 < n; ++i) {
        const double h = x[i + 1] - x[i];
        d[i] = (y[i + 1] - y[i]) / h - h * (2. * m[i] + m[i + 1]) / 6.;
    }
    const double h = x[n - 1] - x[n - 2];
    d[n - 1] = (y[n - 1] - y[n - 2]) / h + h * (m[n - 2] + 2. * m[n - 1]) / 6.;
    return d;
}

// Cubic p(t) on [0, h] with p(0) = f0, p(h) = f1, p'(0) = d0, p'(h) = d1: monomial coefficients as
// rows of H applied to (f0, f1, d0, d1).
static void HermiteMatrix(double h, double H[4][4]) {
    const double ih = 1. / h, ih2 = ih * ih;
    const double rows[4][4] = {{1., 0., 0., 0.},
                               {0., 0., 1., 0.},
                               {-3. * ih2, 3. * ih2, -2. * ih, -ih},
                               {2. * ih2 * ih, -2. * ih2 * ih, ih2, ih2}};
    for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) H[a][b] = rows[a][b];
}

// Knot descriptor with the bucket table of BuildCubic for a general grid (device pointers unset).
static GridDev MakeGrid(const std::vector<double>& x, std::vector<int32_t>& bk) {
    const size_t n = x.size();
    GridDev g;
    g.n = (int32_t)n;
    g.x0 = x.front();
    g.x1 = x.back();
    const int nb = (int)std::min<size_t>(4 * n, 1u << 20);
    g.n_bucket = nb;
    g.inv_dx = nb / (x.back() - x.front());
    bk.assign(nb, 0);
    size_t i = 0;
    for (int j = 0; j < nb; ++j) {
        const double xl = x.front() + j / g.inv_dx;
        while (i + 2 < n && x[i + 1] <= xl) ++i;
        bk[j] = (int32_t)i;
    }
    return g;
}

// Natural bicubic spline through f(x_i, y_j) = f[i n_y + j]. The tensor product of natural cubic
// splines restricted to a cell is the bicubic Hermite polynomial of its corner values f, df/dx,
// df/dy and d2f/dxdy, where df/dx at the knots is the slope of each row's natural spline, df/dy
// that of each column's, and d2f/dxdy the y-slope of the column spline through the row slopes.
BicubicTable Context::BuildBicubic(const std::vector<double>& x, const std::vector<double>& y, const std::vector<double>& f) {
    const size_t nx = x.size(), ny = y.size();
    if (nx < 2 || ny < 2 || f.size() != nx * ny) throw PimcError(kErrInput, "2-D spline needs a full grid of at least 2 x 2 knots");
    for (size_t i = 1; i < nx; ++i)
        if (!(x[i] > x[i - 1])) throw PimcError(kErrInput, "spline knots must increase");
    for (size_t j = 1; j < ny; ++j)
        if (!(y[j] > y[j - 1])) throw PimcError(kErrInput, "spline knots must increase");
    std::vector<double> fx(nx * ny), fy(nx * ny), fxy(nx * ny), line;
    for (size_t j = 0; j < ny; ++j) {  // slopes along x of every row
        line.resize(nx);
        for (size_t i = 0; i < nx; ++i) line[i] = f[i * ny + j];
        const std::vector<double> d = NaturalSlopes(x, line);
        for (size_t i = 0; i < nx; ++i) fx[i * ny + j] = d[i];
    }
    for (size_t i = 0; i < nx; ++i) {  // slopes along y of every column, and of the row slopes
        const std::vector<double> col(f.begin() + i * ny, f.begin() + (i + 1) * ny);
        const std::vector<double> dcol(fx.begin() + i * ny, fx.begin() + (i + 1) * ny);
        const std::vector<double> d = NaturalSlopes(y, col), dd = NaturalSlopes(y, dcol);
        for (size_t j = 0; j < ny; ++j) {
            fy[i * ny + j] = d[j];
            fxy[i * ny + j] = dd[j];
        }
    }
    std::vector<double> c((nx - 1) * (ny - 1) * 16);
    for (size_t i = 0; i + 1 < nx; ++i)
        for (size_t j = 0; j + 1 < ny; ++j) {
            double Hx[4][4], Hy[4][4];
            HermiteMatrix(x[i + 1] - x[i], Hx);
            HermiteMatrix(y[j + 1] - y[j], Hy);
            const size_t a0 = i * ny + j, a1 = (i + 1) * ny + j;
            const double G[4][4] = {{f[a0], f[a0 + 1], fy[a0], fy[a0 + 1]},
                                    {f[a1], f[a1 + 1], fy[a1], fy[a1 + 1]},
                                    {fx[a0], fx[a0 + 1], fxy[a0], fxy[a0 + 1]},
                                    {fx[a1], fx[a1 + 1], fxy[a1], fxy[a1 + 1]}};
            double T[4][4];  // Hx G
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) {
                    double t = 0.;
                    for (int k = 0; k < 4; ++k) t += Hx[a][k] * G[k][b];
                    T[a][b] = t;
                }
            double* cell = &c[(i * (ny - 1) + j) * 16];
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < 4; ++b) {  // (Hx G Hy^T)[a][b]
                    double t = 0.;
                    for (int k = 0; k < 4; ++k) t += T[a][k] * Hy[b][k];
                    cell[4 * a + b] = t;
                }
        }
    BicubicTable t;
    HostBicubic hb;
    t.gx = MakeGrid(x, hb.bx);
    t.gx.x = Upload(x);
    t.gx.bucket = Upload(hb.bx);
    t.gy = MakeGrid(y, hb.by);
    t.gy.x = Upload(y);
    t.gy.bucket = Upload(hb.by);
    t.c = Upload(c);
    hb.x = x;
    hb.y = y;
    hb.c = c;
    host_bicubics.push_back({t.c, hb});
    return t;
}

// Natural cubic splines of several components on one grid, interleaved per interval.
MultiCubic Context::BuildMultiCubic(const std::vector<double>& x, const std::vector<std::vector<double>>& comps) {
    const size_t n = x.size(), nc = comps.size();
    if (n < 2 || nc == 0) throw PimcError(kErrInput, "multi-spline needs at least two knots and one component");
    for (size_t i = 1; i < n; ++i)
        if (!(x[i] > x[i - 1])) throw PimcError(kErrInput, "spline knots must increase");
    std::vector<Cubic4> c((n - 1) * nc);
    for (size_t m = 0; m < nc; ++m) {
        const std::vector<double>& y = comps[m];
        if (y.size() != n) throw PimcError(kErrInput, "multi-spline component of the wrong length");
        const std::vector<double> mm = NaturalSecond(x, y);
        for (size_t i = 0; i + 1 < n; ++i) {
            const double h = x[i + 1] - x[i];
            Cubic4& q = c[i * nc + m];
            q.c0 = y[i];
            q.c1 = (y[i + 1] - y[i]) / h - h * (2. * mm[i] + mm[i + 1]) / 6.;
            q.c2 = 0.5 * mm[i];
            q.c3 = (mm[i + 1] - mm[i]) / (6. * h);
        }
    }
    MultiCubic t;
    std::vector<int32_t> bk;
    t.g = MakeGrid(x, bk);
    t.g.x = Upload(x);
    t.g.bucket = Upload(bk);
    t.c = Upload(c);
    t.n_comp = (int32_t)nc;
    host_multis.push_back({t.c, HostMulti{x, c, bk, (int32_t)nc}});
    return t;
}

// FreeSpline (src/actions/free_spline_class.h:25-68): periodic-image part of the free-particle
// action on a 10000-point uniform grid spanning one box length (1000 for open boundaries).
void Context::FreeSplineTable(double L, uint32_t n_images, double lambda, double tau, bool want_dtau, CubicTable* image,
                              CubicTable* dtau) {
    const double i4lt = 1. / (4. * lambda * tau);
    const double t_l = L == 0. ? 1000. : L;
    const uint32_t num = 10000;
    const double start = -t_l / 2., end = t_l / 2., dr = (end - start) / (num - 1);
    std::vector<double> xs(num), ia(num, 0.), dia(num, 0.);
    for (uint32_t i = 0; i < num; ++i) {
        const double r = start + i * dr;
        xs[i] = r;
        const double r2 = r * r * i4lt;
        for (uint32_t im = 1; im <= n_images; ++im) {
            const double rp = r + im * t_l, rm = r - im * t_l;
            const double dp = r2 - rp * rp * i4lt, dm = r2 - rm * rm * i4lt;
            const double ep = std::exp(dp), em = std::exp(dm);
            ia[i] += ep + em;
            if (want_dtau) dia[i] += (dp * ep + dm * em) / tau;
        }
        if (want_dtau) dia[i] = dia[i] / (1. + ia[i]);
        ia[i] = -std::log1p(ia[i]);
    }
    *image = BuildCubic(xs, ia, true);
    if (want_dtau) *dtau = BuildCubic(xs, dia, true);
}

void Context::BuildPath(const Input& in) {
    Input sysin = in.GetChild("System");
    if (sysin.IsNull()) throw PimcError(kErrInput, "input has no <System> element");
    sys.n_d = sysin.GetAttribute<uint32_t>("n_d");
    sys.M = sysin.GetAttribute<uint32_t>("n_bead");
    sys.beta = sysin.GetAttribute<double>("beta");
    sys.pbc = sysin.GetAttribute<bool>("pbc", true) ? 1 : 0;
    sys.L = sysin.GetAttribute<double>("L", 0.);
    if (sys.n_d < 1 || sys.n_d > 3) throw PimcError(kErrInput, "n_d must be 1, 2 or 3");
    if (sys.M < 2) throw PimcError(kErrInput, "n_bead must be at least 2");
    if (!(sys.beta > 0.)) throw PimcError(kErrInput, "beta must be positive");
    if (sys.pbc) {
        if (!(sys.L > 0.)) throw PimcError(kErrInput, "pbc=1 needs a positive L");
        sys.iL = 1. / sys.L;
        sys.vol = std::pow(sys.L, sys.n_d);
    } else {
        sys.L = 0.;
        sys.iL = 0.;
        sys.vol = 1.;
    }
    sys.tau = sys.beta / (1. * sys.M);
    for (auto& s : in.GetChild("Particles").GetChildList("Species")) {
        if (sys.S >= (uint32_t)kMaxSpecies) throw PimcError(kErrUnsupported, "too many species");
        const uint32_t n = s.GetAttribute<uint32_t>("n_part");
        const double lam = s.GetAttribute<double>("lambda");
        if (n == 0) throw PimcError(kErrInput, "species with n_part = 0");
        // Fermions are sampled as bosons and measured with the permutation sign (Species::GetSign,
        // species_class.h:149-157); the fixed-node restriction needs the nodal actions, which are not built.
        if (s.GetAttribute<bool>("fixed_node", false))
            throw PimcError(kErrUnsupported, "fixed-node species are not supported (no nodal actions)");
        species_fermi.push_back(s.GetAttribute<bool>("fermi", false) ? 1 : 0);
        species_names.push_back(s.GetAttribute<std::string>("name"));
        if (s.GetAttribute<std::string>("init_type", "") == "Restart") {
            // species_class.h:336-345: <prefix>.<proc>.h5 in the reference; the table container here
            std::string file = s.GetAttribute<std::string>("prefix") + "." +
                               std::to_string(s.GetAttribute<bool>("parallel", false) ? chain : 0u) + ".pat";
            if (!file.empty() && file[0] != '/' && !base_dir.empty()) file = base_dir + "/" + file;
            restarts.push_back(RestartSpec{sys.S, file, s.GetAttribute<std::string>("path_dump_name", "path_dump")});
        }
        sys.sp_off[sys.S] = sys.n_total;
        sys.sp_n[sys.S] = n;
        sys.sp_lambda[sys.S] = lam;
        sys.sp_rho[sys.S] = -1;
        sys.n_total += n;
        sys.S++;
    }
    if (sys.S == 0) throw PimcError(kErrInput, "input declares no species");
    sys.n_pad = (sys.n_total + 31u) & ~31u;
    pos_.reset(new DeviceBuffer((size_t)sys.M * 3 * sys.n_pad * sizeof(double)));
    pos_new_.reset(new DeviceBuffer((size_t)sys.M * 3 * sys.n_pad * sizeof(double)));
    sys.pos = pos_->as<double>();
    sys.pos_new = pos_new_->as<double>();
    perm_.reset(new DeviceBuffer(sys.n_total * sizeof(uint32_t)));
    perm_inv_.reset(new DeviceBuffer(sys.n_total * sizeof(uint32_t)));
    perm_host.resize(sys.n_total);
    for (uint32_t g = 0; g < sys.n_total; ++g) perm_host[g] = g;
    CudaCheck(cudaMemcpy(perm_->ptr, perm_host.data(), sys.n_total * sizeof(uint32_t), cudaMemcpyHostToDevice), "perm upload");
    CudaCheck(cudaMemcpy(perm_inv_->ptr, perm_host.data(), sys.n_total * sizeof(uint32_t), cudaMemcpyHostToDevice), "perm upload");
    sys.perm = perm_->as<uint32_t>();
    sys.perm_inv = perm_inv_->as<uint32_t>();
}

static uint32_t SpeciesIndex(const std::vector<std::string>& names, const std::string& n) {
    for (size_t i = 0; i < names.size(); ++i)
        if (names[i] == n) return (uint32_t)i;
    throw PimcError(kErrInput, "no species named '" + n + "'");
}

namespace {

// KSpace::Include / Setup (k_space_class.h:17-80); lexicographic enumeration of the index box.
struct KSet {
    double cutoff = 0.;
    int max_index[3] = {0, 0, 0};
    std::vector<std::vector<int>> n;
    std::vector<double> mags;

    void Setup(double k_cut, double L, uint32_t n_d) {
        if (L == 0. || k_cut <= cutoff) return;
        cutoff = k_cut;
        n.clear();
        mags.clear();
        const double box = 2. * M_PI / L;
        for (uint32_t d = 0; d < n_d; ++d) max_index[d] = (int)(uint32_t)std::ceil(1.1 * k_cut / box);
        std::vector<int> v(n_d);
        for (uint32_t d = 0; d < n_d; ++d) v[d] = -max_index[d];
        for (;;) {
            double k[3] = {0., 0., 0.}, k2 = 0.;
            for (uint32_t d = 0; d < n_d; ++d) {
                k[d] = v[d] * box;
                k2 += k[d] * k[d];
            }
            bool inc = false;
            if (k2 < k_cut * k_cut && k2 != 0.) {
                if (k[0] > 0.) inc = true;
                else if (n_d >= 2 && k[0] == 0. && k[1] > 0.) inc = true;
                else if (n_d >= 3 && k[0] == 0. && k[1] == 0. && k[2] > 0.) inc = true;
            }
            if (inc) {
                n.push_back(v);
                mags.push_back(std::sqrt(k2));
            }
            int d = (int)n_d - 1;
            while (d >= 0) {
                if (++v[d] <= max_index[d]) break;
                v[d] = -max_index[d];
                --d;
            }
            if (d < 0) break;
        }
    }
};

}  // namespace

void Context::BuildActions(const Input& in) {
    // k-space: the System cutoff, then every long-range action and structure factor may raise it
    // (path_class.h:58-62, pair_action_class.h:216-222, structure_factor_class.h:49-54).
    KSet ks;
    Input sysin = in.GetChild("System");
    if (sys.pbc) ks.Setup(sysin.GetAttribute<double>("k_cut", 2. * M_PI / sys.L), sys.L, sys.n_d);
    auto alist = in.GetChild("Actions").GetChildList("Action");
    bool long_range_seen = false;
    for (const auto& a : alist) {
        const std::string ty = a.GetAttribute<std::string>("type");
        if ((ty == "BarePairAction" || ty == "IlkkaPairAction" || ty == "DavidPairAction") && a.GetAttribute<bool>("use_long_range", false)) {
            if (!sys.pbc) throw PimcError(kErrInput, "use_long_range needs periodic boundaries");
            const double before = ks.cutoff;
            ks.Setup(a.GetAttribute<double>("k_cut", ks.cutoff), sys.L, sys.n_d);
            // A later, larger cutoff would outgrow the tables of earlier long-range actions.
            if (long_range_seen && ks.cutoff != before)
                throw PimcError(kErrInput, "k_cut of a long-range action grows after an earlier one; order the largest first");
            long_range_seen = true;
        }
    }
    for (auto& o : in.GetChild("Observables").GetChildList("Observable"))
        if (o.GetAttribute<std::string>("type") == "StructureFactor") {
            if (!sys.pbc) throw PimcError(kErrInput, "StructureFactor needs periodic boundaries");
            const double before = ks.cutoff;
            ks.Setup(o.GetAttribute<double>("k_cut", ks.cutoff), sys.L, sys.n_d);
            if (long_range_seen && ks.cutoff != before)
                throw PimcError(kErrInput, "StructureFactor k_cut exceeds a long-range action's k_cut");
        }
    kcutoff = ks.cutoff;
    sys.K = (uint32_t)ks.n.size();
    for (int d = 0; d < 3; ++d) sys.max_index[d] = ks.max_index[d];
    for (uint32_t d = 0; d < 3; ++d) sys.box[d] = sys.pbc ? 2. * M_PI / sys.L : 0.;
    kmags = ks.mags;
    kint = ks.n;
    std::vector<int32_t> packed(sys.K);
    for (uint32_t k = 0; k < sys.K; ++k) {
        int v[3] = {0, 0, 0};
        for (uint32_t d = 0; d < sys.n_d; ++d) v[d] = ks.n[k][d];
        if (std::abs(v[0]) > 127 || std::abs(v[1]) > 127 || std::abs(v[2]) > 127) throw PimcError(kErrUnsupported, "k index beyond 127");
        packed[k] = PackK(v[0], v[1], v[2]);
    }
    if (sys.K) sys.kidx = Upload(packed);

    for (auto& a : alist) {
        ActionHost h;
        h.name = a.GetAttribute<std::string>("name");
        h.type = a.GetAttribute<std::string>("type");
        const int n_images = a.GetAttribute<int>("n_images", 0);
        const uint32_t max_level = a.GetAttribute<uint32_t>("max_level", 0);
        if (h.type == "Kinetic") {
            if (sys.n_kinetic >= kMaxKinetic) throw PimcError(kErrUnsupported, "too many kinetic actions");
            KineticDev& k = sys.kinetic[sys.n_kinetic];
            k.species = SpeciesIndex(species_names, a.GetAttribute<std::string>("species"));
            const double lam = sys.sp_lambda[k.species];
            if (!(lam > 0.)) throw PimcError(kErrInput, "Kinetic action on a species with lambda = 0");
            k.has_images = n_images > 0 ? 1 : 0;
            k.i4lt = 1. / (4. * lam * sys.tau);
            k.i4ltt = 1. / (4. * lam * sys.tau * sys.tau);
            k.d_action_d_beta_const = sys.sp_n[k.species] * sys.M * sys.n_d / (2. * sys.tau);
            // kinetic_class.h:16-24: spline i holds tau (i + 1); the bisection uses skip = 2^l.
            const uint32_t n_spline = sys.M / 2 + (sys.M % 2) + 1;
            for (int l = 0; l < kMaxLevels && (1u << l) <= n_spline; ++l) {
                k.i4lt_level[l] = 1. / (4. * lam * (sys.tau * (1u << l)));
                FreeSplineTable(sys.L, (uint32_t)std::max(n_images, 0), lam, sys.tau * (1u << l), l == 0, &k.image[l],
                                l == 0 ? &k.d_image_d_tau : nullptr);
            }
            h.kind = 0;
            h.index = sys.n_kinetic++;
            h.species_list.push_back(k.species);
        } else if (h.type == "HarmonicTrap") {
            if (sys.n_trap >= kMaxTrap) throw PimcError(kErrUnsupported, "too many trap actions");
            TrapDev& t = sys.trap[sys.n_trap];
            t.species = SpeciesIndex(species_names, a.GetAttribute<std::string>("species"));
            t.max_level = max_level;
            const double om = a.GetAttribute<double>("omega");
            t.cofactor_a = 0.5 * sys.tau * om * om * (1. + sys.tau * sys.tau * om * om / 12.);
            t.cofactor_b = 0.5 * om * om * (1. + 3. * sys.tau * sys.tau * om * om / 12.);
            h.kind = 1;
            h.index = sys.n_trap++;
            h.species_list.push_back(t.species);
        } else if (h.type == "BarePairAction") {
            if (sys.n_pair >= kMaxPair) throw PimcError(kErrUnsupported, "too many pair actions");
            PairDev& p = sys.pair[sys.n_pair];
            p.sa = SpeciesIndex(species_names, a.GetAttribute<std::string>("species_a"));
            p.sb = SpeciesIndex(species_names, a.GetAttribute<std::string>("species_b"));
            p.max_level = max_level;
            p.use_long_range = a.GetAttribute<bool>("use_long_range", false) ? 1 : 0;
            p.is_coulomb = a.GetAttribute<bool>("is_coulomb", false) ? 1 : 0;
            p.is_constant = (p.sa == p.sb) && (sys.sp_n[p.sa] == 1 || sys.sp_lambda[p.sa] == 0.);
            std::string file = a.GetAttribute<std::string>("file");
            if (!file.empty() && file[0] != '/' && !base_dir.empty()) file = base_dir + "/" + file;
            TableFile tf = TableFile::Load(file);
            const auto& r = tf.Vec("v/diag/r");
            const auto& v = tf.Vec("v/diag/v_r");
            if ((size_t)tf.Scalar("v/diag/n_r") != r.size() || r.size() != v.size())
                throw PimcError(kErrInput, "table '" + file + "': inconsistent v/diag grid");
            p.v_r = BuildCubic(r, v, false);
            p.r_v_min = r.front();
            p.r_v_max = r.back();
            double vk0 = 0., vr0 = 0.;
            if (p.use_long_range) {
                const auto& rl = tf.Vec("v/diag/r_long");
                const auto& vl = tf.Vec("v/diag/v_long_r");
                vr0 = tf.Scalar("v/diag/v_long_r_0");
                p.v_long_r = BuildCubic(rl, vl, false);
                p.r_vl_min = rl.front();
                p.r_vl_max = rl.back();
                const auto& kv = tf.Vec("v/diag/k");
                const auto& vkv = tf.Vec("v/diag/v_long_k");
                vk0 = tf.Scalar("v/diag/v_long_k_0");
                // bare_pair_action_class.h:79-85: match every stored |k| against the table.
                std::vector<double> vk(sys.K, 0.);
                for (uint32_t k = 0; k < sys.K; ++k)
                    for (size_t j = 0; j < kv.size(); ++j)
                        if (std::fabs(kmags[k] - kv[j]) < 1.e-8) vk[k] = vkv[j];
                p.v_long_k = Upload(vk);
                host_vk.resize(sys.n_pair + 1);
                host_vk[sys.n_pair] = vk;
                sys.sp_rho[p.sa] = sys.sp_rho[p.sb] = 0;  // marked; slots assigned below
            }
            // bare_pair_action_class.h:89-95
            if (p.sa == p.sb) {
                vk0 *= 0.5 * sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                vr0 *= -0.5 * sys.sp_n[p.sa] * sys.M;
            } else {
                vk0 *= (double)sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                vr0 *= 0.;
            }
            p.v_long_k_0 = vk0;
            p.v_long_r_0 = vr0;
            h.kind = 2;
            h.index = sys.n_pair++;
            h.species_list.push_back(p.sa);
            h.species_list.push_back(p.sb);
        } else if (h.type == "DavidPairAction") {
            // david_pair_action_class.h:190-358
            if (sys.n_pair >= kMaxPair) throw PimcError(kErrUnsupported, "too many pair actions");
            PairDev& p = sys.pair[sys.n_pair];
            p.kind = kPairDavid;
            p.sa = SpeciesIndex(species_names, a.GetAttribute<std::string>("species_a"));
            p.sb = SpeciesIndex(species_names, a.GetAttribute<std::string>("species_b"));
            p.max_level = max_level;
            p.use_long_range = a.GetAttribute<bool>("use_long_range", false) ? 1 : 0;
            p.is_coulomb = 0;
            p.is_constant = (p.sa == p.sb) && (sys.sp_n[p.sa] == 1 || sys.sp_lambda[p.sa] == 0.);
            p.n_order = a.GetAttribute<uint32_t>("n_order", 0);  // pair_action_class.h:208
            std::string file = a.GetAttribute<std::string>("file");
            if (!file.empty() && file[0] != '/' && !base_dir.empty()) file = base_dir + "/" + file;
            TableFile tf = TableFile::Load(file);
            const std::string pre = "u_kj_" + std::to_string(p.n_order), dpre = "du_kj_dbeta_" + std::to_string(p.n_order);
            const auto& grid = tf.Vec(pre + "/grid/grid_points");
            const size_t n_grid = grid.size();
            if ((size_t)tf.Scalar(pre + "/grid/n_grid_points") != n_grid || n_grid < 2)
                throw PimcError(kErrInput, "table '" + file + "': inconsistent grid");
            // :234-246: n_tau = max_level + 1 tables; the path's tau must be among the first n_tau taus,
            // and level l reads table l whatever its tau.
            const size_t n_tau = (size_t)max_level + 1;
            const auto& taus = tf.Vec(pre + "/taus");
            if (taus.size() < n_tau) throw PimcError(kErrInput, "table '" + file + "': fewer taus than max_level + 1");
            bool found = false;
            for (size_t i = 0; i < n_tau; ++i) found |= std::fabs(taus[i] - sys.tau) < 1.0e-6;
            if (!found) throw PimcError(kErrInput, "table '" + file + "': tau of the path not found");
            const auto& V = tf.Vec("potential/data");
            uint32_t n_val = 1;
            for (uint32_t i = 1; i <= p.n_order; ++i) n_val += 1 + i;
            p.kj_stride = n_val + 1;
            // Value index fastest, then grid, then tau. The reference fills its spline data for the
            // grid points below the last one only (david_pair_action_class.h:262-271, the zeroing of
            // the last one commented out); its array library zero-initialises, so every component,
            // the potential included, is zero at the last grid point.
            auto comps = [&](const std::string& key) {
                const auto& d = tf.Vec(key);
                if (d.size() < (size_t)n_val * n_grid * n_tau || V.size() != n_grid)
                    throw PimcError(kErrInput, "table '" + file + "': short " + key);
                std::vector<std::vector<double>> out(n_tau * (n_val + 1), std::vector<double>(n_grid, 0.));
                for (size_t l = 0; l < n_tau; ++l)
                    for (size_t g = 0; g + 1 < n_grid; ++g) {
                        out[l * (n_val + 1)][g] = V[g];
                        for (uint32_t v = 1; v <= n_val; ++v) out[l * (n_val + 1) + v][g] = d[(v - 1) + g * n_val + l * n_val * n_grid];
                    }
                return out;
            };
            p.u_kj = BuildMultiCubic(grid, comps(pre + "/data"));
            p.du_kj = BuildMultiCubic(grid, comps(dpre + "/data"));
            p.r_d_min = grid.front();
            p.r_d_max = grid.back();
            double vk0 = 0., vr0 = 0.;
            if (p.use_long_range) {
                const auto& kv = tf.Vec("long_range/k_points");
                const auto& ukv = tf.Vec("long_range/u_k");
                std::vector<double> uk(sys.K, 0.), duk(sys.K, 0.), vk(sys.K, 0.);
                for (size_t i = 0; i < kv.size() && i < ukv.size(); ++i) {
                    const double v = ukv[i] / sys.vol;
                    if (std::fabs(kv[i]) < 1.e-8) vk0 = v;
                    for (uint32_t k = 0; k < sys.K; ++k)
                        if (std::fabs(kmags[k] - kv[i]) < 1.e-8) {
                            uk[k] = v * sys.tau;
                            duk[k] = v;
                            vk[k] = v;
                        }
                }
                vr0 = tf.Scalar("squarer/v_image");
                p.u_long_k = Upload(uk);
                p.du_long_k = Upload(duk);
                p.v_long_k = Upload(vk);
                host_vk.resize(sys.n_pair + 1);
                host_vk[sys.n_pair] = vk;  // u_long_k / tau
                sys.sp_rho[p.sa] = sys.sp_rho[p.sb] = 0;  // marked; slots assigned below
            }
            double dk0 = vk0, dr0 = vr0;
            if (p.sa == p.sb) {  // :340-356
                dk0 *= 0.5 * sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                dr0 *= -0.5 * sys.sp_n[p.sa] * sys.M;
                vk0 *= 0.5 * sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                vr0 *= -0.5 * sys.sp_n[p.sa] * sys.M;
            } else {
                dk0 *= (double)sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                dr0 *= 0.;
                vk0 *= (double)sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                vr0 *= 0.;
            }
            p.du_long_k_0 = dk0;
            p.du_long_r_0 = dr0;
            p.v_long_k_0 = vk0;
            p.v_long_r_0 = vr0;
            h.kind = 2;
            h.index = sys.n_pair++;
            h.species_list.push_back(p.sa);
            h.species_list.push_back(p.sb);
        } else if (h.type == "IlkkaPairAction") {
            // ilkka_pair_action_class.h:253-432
            if (sys.n_pair >= kMaxPair) throw PimcError(kErrUnsupported, "too many pair actions");
            PairDev& p = sys.pair[sys.n_pair];
            p.kind = kPairIlkka;
            p.sa = SpeciesIndex(species_names, a.GetAttribute<std::string>("species_a"));
            p.sb = SpeciesIndex(species_names, a.GetAttribute<std::string>("species_b"));
            p.max_level = max_level;
            p.use_long_range = a.GetAttribute<bool>("use_long_range", false) ? 1 : 0;
            p.is_coulomb = 0;
            p.is_constant = (p.sa == p.sb) && (sys.sp_n[p.sa] == 1 || sys.sp_lambda[p.sa] == 0.);
            std::string file = a.GetAttribute<std::string>("file");
            if (!file.empty() && file[0] != '/' && !base_dir.empty()) file = base_dir + "/" + file;
            TableFile tf = TableFile::Load(file);
            auto grid2 = [&](const std::string& g, const std::string& f) {
                const auto& x = tf.Vec(g + "/off_diag/x");
                const auto& y = tf.Vec(g + "/off_diag/y");
                if ((size_t)tf.Scalar(g + "/off_diag/n_x") != x.size() || (size_t)tf.Scalar(g + "/off_diag/n_y") != y.size())
                    throw PimcError(kErrInput, "table '" + file + "': inconsistent " + g + "/off_diag grid");
                return BuildBicubic(x, y, tf.Vec(g + "/off_diag/" + f));
            };
            // Each stored k-vector takes the table value of its magnitude (:308-315).
            auto by_mag = [&](const std::string& kd, const std::string& vd) {
                const auto& kv = tf.Vec(kd);
                const auto& vv = tf.Vec(vd);
                std::vector<double> out(sys.K, 0.);
                for (uint32_t k = 0; k < sys.K; ++k)
                    for (size_t j = 0; j < kv.size() && j < vv.size(); ++j)
                        if (std::fabs(kmags[k] - kv[j]) < 1.e-8) out[k] = vv[j];
                return out;
            };
            p.u_xy = grid2("u", "u_xy");
            p.du_xy = grid2("du", "du_xy");
            {
                const auto& r = tf.Vec("v/diag/r");
                const auto& v = tf.Vec("v/diag/v_r");
                if ((size_t)tf.Scalar("v/diag/n_r") != r.size() || r.size() != v.size())
                    throw PimcError(kErrInput, "table '" + file + "': inconsistent v/diag grid");
                p.v_r = BuildCubic(r, v, false);
                p.r_v_min = r.front();
                p.r_v_max = r.back();
            }
            double vk0 = 0., vr0 = 0., dk0 = 0., dr0 = 0.;
            if (p.use_long_range) {
                const auto& ru = tf.Vec("u/diag/r_long");
                p.u_long_r = BuildCubic(ru, tf.Vec("u/diag/u_long_r"), false);
                p.r_u_min = ru.front();
                p.r_u_max = ru.back();
                const auto& rd = tf.Vec("du/diag/r_long");
                p.du_long_r = BuildCubic(rd, tf.Vec("du/diag/du_long_r"), false);
                p.r_du_min = rd.front();
                p.r_du_max = rd.back();
                dr0 = tf.Scalar("du/diag/du_long_r_0");
                dk0 = tf.Scalar("du/diag/du_long_k_0");
                const auto& rv = tf.Vec("v/diag/r_long");
                p.v_long_r = BuildCubic(rv, tf.Vec("v/diag/v_long_r"), false);
                p.r_vl_min = rv.front();
                p.r_vl_max = rv.back();
                vr0 = tf.Scalar("v/diag/v_long_r_0");
                vk0 = tf.Scalar("v/diag/v_long_k_0");
                const std::vector<double> uk = by_mag("u/diag/k", "u/diag/u_long_k");
                p.u_long_k = Upload(uk);
                p.du_long_k = Upload(by_mag("du/diag/k", "du/diag/du_long_k"));
                p.v_long_k = Upload(by_mag("v/diag/k", "v/diag/v_long_k"));
                // The sweep multiplies every long-range coefficient by tau.
                std::vector<double> scaled(uk);
                for (auto& x : scaled) x /= sys.tau;
                host_vk.resize(sys.n_pair + 1);
                host_vk[sys.n_pair] = scaled;
                sys.sp_rho[p.sa] = sys.sp_rho[p.sb] = 0;  // marked; slots assigned below
            }
            if (p.sa == p.sb) {  // :420-431
                dk0 *= 0.5 * sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                dr0 *= -0.5 * sys.sp_n[p.sa] * sys.M;
                vk0 *= 0.5 * sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                vr0 *= -0.5 * sys.sp_n[p.sa] * sys.M;
            } else {
                dk0 *= (double)sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                dr0 *= 0.;
                vk0 *= (double)sys.sp_n[p.sa] * sys.sp_n[p.sb] * sys.M;
                vr0 *= 0.;
            }
            p.du_long_k_0 = dk0;
            p.du_long_r_0 = dr0;
            p.v_long_k_0 = vk0;
            p.v_long_r_0 = vr0;
            h.kind = 2;
            h.index = sys.n_pair++;
            h.species_list.push_back(p.sa);
            h.species_list.push_back(p.sb);
        } else {
            throw PimcError(kErrUnsupported, "unsupported action type '" + h.type + "'");
        }
        actions.push_back(h);
    }
}

void Context::BuildMoves(const Input& in) {
    for (auto& m : in.GetChild("Moves").GetChildList("Move")) {
        MoveHost h;
        h.name = m.GetAttribute<std::string>("name");
        h.type = m.GetAttribute<std::string>("type");
        if (moves.size() >= (size_t)kMaxMoves) throw PimcError(kErrUnsupported, "too many moves");
        if (h.type == "HMC") {
            // Hybrid Monte Carlo of the whole path (no reference counterpart).
            h.kind = 1;
            h.hmc_step = m.GetAttribute<double>("step_size", 0.01);
            h.hmc_steps = m.GetAttribute<uint32_t>("n_steps", 10);
            const std::string sp = m.GetAttribute<std::string>("species", "");
            h.hmc_species = sp.empty() ? -1 : (int)SpeciesIndex(species_names, sp);
            if (!(h.hmc_step > 0.) || h.hmc_steps == 0) throw PimcError(kErrInput, "HMC needs step_size > 0 and n_steps > 0");
            moves.push_back(h);
            continue;
        }
        if (h.type == "PermBisectIterative") h.kind = 2;
        else if (h.type == "PermBisectTable") h.kind = 3;
        else if (h.type != "Bisect") throw PimcError(kErrUnsupported, "unsupported move type '" + h.type + "'");
        MoveDev& d = h.dev;
        d.species = SpeciesIndex(species_names, m.GetAttribute<std::string>("species"));
        d.n_level = m.GetAttribute<uint32_t>("n_level");
        d.lambda = sys.sp_lambda[d.species];
        if (!(d.lambda > 0.)) throw PimcError(kErrInput, "Bisect on a species with lambda = 0");
        if (d.n_level < 1 || (1u << d.n_level) > sys.M || d.n_level > (uint32_t)kMaxLevels)
            throw PimcError(kErrInput, "bisection level out of range for n_bead");
        const int n_images = m.GetAttribute<int>("n_images", 0);
        d.has_images = n_images > 0 ? 1 : 0;
        h.adaptive = m.GetAttribute<bool>("adaptive", false);
        if (h.adaptive) h.target_ratio = m.GetAttribute<double>("target_ratio");
        // bisect_class.h:158-163: sampling propagator at tau' = tau 2^l / 2.
        const uint32_t n_spline = (uint32_t)std::floor(std::log2((double)sys.M));
        for (uint32_t l = 0; l < n_spline && l < (uint32_t)kMaxLevels; ++l) {
            const double tl = 0.5 * sys.tau * (1u << l);
            d.i4lt_sample[l] = 1. / (4. * d.lambda * tl);
            if (d.has_images) FreeSplineTable(sys.L, (uint32_t)n_images, d.lambda, tl, false, &d.sample_image[l], nullptr);
        }
        // move_class.h:27-31: every action whose species list holds the move's species.
        for (auto& a : actions) {
            if (std::find(a.species_list.begin(), a.species_list.end(), d.species) == a.species_list.end()) continue;
            if (a.kind == 0) d.kinetic[d.n_kinetic++] = a.index;
            else if (a.kind == 1) d.trap[d.n_trap++] = a.index;
            else d.pair[d.n_pair++] = a.index;
        }
        if (h.kind == 2 || h.kind == 3) {
            // perm_bisect_class.h:101-116
            const uint32_t N = sys.sp_n[d.species];
            h.perm_epsilon = m.GetAttribute<double>("epsilon", 1.e-100);
            h.perm_attempt.assign(N, 0);
            h.perm_accept.assign(N, 0);
            h.perm_n_type_out = N;  // perm_bisect_iterative_class.h:229
            if (h.kind == 3) {
                // BuildCycles (perm_bisect_table_class.h:54-102): every permutation of n_perm_part
                // particles (lexicographic) over every subset of that size (lexicographic).
                const uint32_t k = m.GetAttribute<uint32_t>("n_perm_part");
                if (k < 1 || k > N) throw PimcError(kErrInput, "n_perm_part must be between 1 and the particle count");
                std::vector<uint32_t> a(k), types, combs;
                for (uint32_t i = 0; i < k; ++i) a[i] = i;
                uint32_t n_types = 0, n_comb = 0;
                do {
                    types.insert(types.end(), a.begin(), a.end());
                    ++n_types;
                } while (std::next_permutation(a.begin(), a.end()));
                std::vector<uint32_t> c(k);
                for (uint32_t i = 0; i < k; ++i) c[i] = i;
                for (;;) {
                    combs.insert(combs.end(), c.begin(), c.end());
                    ++n_comb;
                    if ((size_t)n_comb * n_types > (1u << 24)) throw PimcError(kErrUnsupported, "permutation table above 2^24 cycles");
                    int i = (int)k - 1;
                    while (i >= 0 && c[i] == N - k + (uint32_t)i) --i;
                    if (i < 0) break;
                    c[i]++;
                    for (uint32_t j = (uint32_t)i + 1; j < k; ++j) c[j] = c[j - 1] + 1;
                }
                h.perm_k = k;
                h.perm_n_types = n_types;
                h.perm_n_comb = n_comb;
                h.perm_n_type_out = n_types;
                h.perm_types = std::make_shared<DeviceBuffer>(types.size() * sizeof(uint32_t));
                h.perm_combs = std::make_shared<DeviceBuffer>(combs.size() * sizeof(uint32_t));
                CudaCheck(cudaMemcpy(h.perm_types->ptr, types.data(), types.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "cycle table upload");
                CudaCheck(cudaMemcpy(h.perm_combs->ptr, combs.data(), combs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice), "cycle table upload");
            }
        }
        moves.push_back(h);
    }
}

void Context::BuildObservables(const Input& in) {
    for (auto& o : in.GetChild("Observables").GetChildList("Observable")) {
        ObservableHost h;
        h.name = o.GetAttribute<std::string>("name");
        h.type = o.GetAttribute<std::string>("type");
        if (h.type == "Energy") {
            h.kind = 0;
            h.measure_potential = o.GetAttribute<bool>("measure_potential", false);
            h.use_virial = o.GetAttribute<bool>("use_virial_estimator", false);
            h.use_adjoint = o.GetAttribute<bool>("use_adjoint_gradient", false);
            if (h.use_virial) {
                h.virial_window = o.GetAttribute<uint32_t>("virial_window_size", sys.M);
                h.use_thermal = o.GetAttribute<bool>("use_thermal_estimator", false);
            } else {
                h.use_thermal = o.GetAttribute<bool>("use_thermal_estimator", true);
            }
            h.energies.assign(actions.size(), 0.);
            h.potentials.assign(actions.size(), 0.);
        } else if (h.type == "PairCorrelation") {
            h.kind = 1;
            h.sa = SpeciesIndex(species_names, o.GetAttribute<std::string>("species_a"));
            h.sb = SpeciesIndex(species_names, o.GetAttribute<std::string>("species_b"));
            h.r_min = o.GetAttribute<double>("r_min", 0.);
            h.r_max = o.GetAttribute<double>("r_max", sys.L / 2.);
            h.n_r = o.GetAttribute<uint32_t>("n_r", 100);
            if (h.n_r < 2) throw PimcError(kErrInput, "n_r must be at least 2");
            h.dr = (h.r_max - h.r_min) / (h.n_r - 1.);
            h.d_ir = 1. / h.dr;
            h.hist.reset(new DeviceBuffer(h.n_r * sizeof(unsigned long long)));
        } else if (h.type == "StructureFactor") {
            h.kind = 2;
            h.sa = SpeciesIndex(species_names, o.GetAttribute<std::string>("species_a"));
            h.sb = SpeciesIndex(species_names, o.GetAttribute<std::string>("species_b"));
            h.k_cut = o.GetAttribute<double>("k_cut", kcutoff);
            sys.sp_rho[h.sa] = sys.sp_rho[h.sb] = 0;
            h.sk.reset(new DeviceBuffer(std::max<size_t>(sys.K, 1) * sizeof(double)));
        } else if (h.type == "PathDump") {
            h.kind = 4;
            h.skip = std::max(1u, o.GetAttribute<uint32_t>("skip", 1));  // observable_class.h:77
            h.dumps.resize(sys.S);
            h.dump_perms.resize(sys.S);
        } else if (h.type == "Time") {
            h.kind = 3;
        } else if (h.type == "Sign") {
            h.kind = 5;
        } else if (h.type == "Permutation") {
            // permutation_class.h:33-73; sectors are the partitions of N in the order of the
            // ascending-composition generation of species_class.h:178-221
            h.kind = 6;
            h.species = SpeciesIndex(species_names, o.GetAttribute<std::string>("species"));
            h.sector_max = o.GetAttribute<uint32_t>("sector_max", 0);
            const uint32_t n = sys.sp_n[h.species];
            h.cycles.assign(n, 0.);
            // Accelerated ascending-composition generation of the partitions of n (Kelleher and
            // O'Sullivan), stopped after sector_max partitions when sector_max > 0.
            std::vector<uint32_t> a(n + 1, 0);
            uint32_t k = 1, y = n - 1;
            auto room = [&]() { return h.sector_max == 0 || h.partitions.size() < h.sector_max; };
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
                    h.partitions.emplace_back(a.begin(), a.begin() + k + 2);
                    x += 1;
                    y -= 1;
                }
                a[k] = x + y;
                y = x + y - 1;
                h.partitions.emplace_back(a.begin(), a.begin() + k + 1);
                if (h.partitions.size() > (1u << 20)) throw PimcError(kErrUnsupported, "more than 2^20 permutation sectors: set sector_max");
            }
        } else {
            throw PimcError(kErrUnsupported, "unsupported observable type '" + h.type + "'");
        }
        observables.push_back(std::move(h));
    }
}

void Context::ReadLoop(const Input& in, LoopNode& node) {
    // loop_class.h:34-52
    for (auto& c : in.GetChildList()) {
        const std::string& t = c.GetName();
        LoopNode ch;
        if (t == "Move" || t == "Observable") {
            const std::string nm = c.GetAttribute<std::string>("name");
            bool found = false;
            if (t == "Move") {
                for (size_t i = 0; i < moves.size(); ++i)
                    if (moves[i].name == nm) { ch.kind = 1; ch.index = (uint32_t)i; found = true; }
            } else {
                for (size_t i = 0; i < observables.size(); ++i)
                    if (observables[i].name == nm) { ch.kind = 2; ch.index = (uint32_t)i; found = true; }
            }
            if (!found) continue;
        } else if (t == "Write") {
            ch.kind = 3;
        } else if (t == "Loop") {
            ch.kind = 0;
            ch.n_steps = (uint64_t)c.GetAttribute<int>("n_step");
            ReadLoop(c, ch);
        } else {
            continue;
        }
        node.children.push_back(std::move(ch));
    }
}

Context::Context(const Input& in, const std::string& bd, int dev, uint32_t ch) : device(dev), chain(ch), base_dir(bd) {
    CudaCheck(cudaSetDevice(device), "cudaSetDevice");
    CudaCheck(cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, device), "device attribute");
    CudaCheck(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "stream create");
    Input rng = in.GetChild("RNG");
    seed = rng.IsNull() ? (uint32_t)time(nullptr) : (uint32_t)rng.GetAttribute<int>("seed", (int)time(nullptr));
    BuildPath(in);
    BuildActions(in);
    BuildMoves(in);
    BuildObservables(in);
    // Charge-density slots for species that need them.
    for (uint32_t s = 0; s < sys.S; ++s)
        if (sys.sp_rho[s] == 0) sys.sp_rho[s] = rho_slots++;
        else sys.sp_rho[s] = -1;
    if (rho_slots && sys.K) {
        rho_.reset(new DeviceBuffer((size_t)rho_slots * sys.M * sys.K * sizeof(double2)));
        sys.rho_k = rho_->as<double2>();
    }
    partials_.reset(new DeviceBuffer(4096 * sizeof(double)));
    partials_cap_ = 4096;
    result_.reset(new DeviceBuffer(64 * sizeof(double)));
    bar_.reset(new DeviceBuffer(64));
    err_.reset(new DeviceBuffer(64));
    blocks.resize(observables.size());
    Input alg = in.GetChild("Algorithm");
    main_loop.kind = 0;
    main_loop.n_steps = 1;
    ReadLoop(alg, main_loop);
    InitRhoK();
    ApplyRestarts();
}

Context::~Context() {
    if (stream) {
        cudaStreamSynchronize(stream);
        cudaStreamDestroy(stream);
    }
}

double* Context::Partials(size_t n) {
    if (n > partials_cap_) {
        partials_.reset(new DeviceBuffer(n * sizeof(double)));
        partials_cap_ = n;
    }
    return partials_->as<double>();
}

uint32_t* Context::Pairs(size_t n_pairs) {
    if (2 * n_pairs > pairs_cap_) {
        pairs_.reset(new DeviceBuffer(2 * n_pairs * sizeof(uint32_t)));
        pairs_cap_ = 2 * n_pairs;
    }
    return pairs_->as<uint32_t>();
}

double2* Context::RhoTmp(size_t n) {
    if (n > rho_tmp_cap_) {
        rho_tmp_.reset(new DeviceBuffer(n * sizeof(double2)));
        rho_tmp_cap_ = n;
    }
    return rho_tmp_->as<double2>();
}

uint32_t* Context::Parts(size_t n) {
    if (n > parts_cap_) {
        parts_.reset(new DeviceBuffer(n * sizeof(uint32_t)));
        parts_cap_ = n;
    }
    return parts_->as<uint32_t>();
}

void Context::Sync() { CudaCheck(cudaStreamSynchronize(stream), "stream synchronize"); }

void Context::CheckDeviceError(bool path_written) {
    int e = 0;
    CudaCheck(cudaMemcpyAsync(&e, err_->ptr, sizeof(int), cudaMemcpyDeviceToHost, stream), "read error word");
    Sync();
    if (e != 0) {
        int zero = 0;
        CudaCheck(cudaMemcpyAsync(err_->ptr, &zero, sizeof(int), cudaMemcpyHostToDevice, stream), "clear error word");
        Sync();
        if (e == kDevErrTimeout) {
            // Blocks that gave up left the launch mid-attempt: some may have committed beads or
            // densities that others did not.
            if (path_written) path_lost = true;
            throw PimcError(kErrTimeout, "device wait timed out (grid barrier)");
        }
        if (e == kDevErrNonFinite) throw PimcError(kErrNonFinite, "non-finite value in the path");
        throw PimcError(kErrState, "device reported error " + std::to_string(e));
    }
}

void Context::RequirePath() const {
    if (path_lost)
        throw PimcError(kErrState, "the path is undefined after a launch that timed out; set it again with pimc_set_path(ctx, 2, ...)");
}

void Context::SetPath(int which, const double* h) {
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    std::vector<double> buf((size_t)M * 3 * np, 0.);
    for (uint32_t g = 0; g < sys.n_total; ++g)
        for (uint32_t b = 0; b < M; ++b)
            for (uint32_t d = 0; d < n_d; ++d) {
                const double v = h[((size_t)g * M + b) * n_d + d];
                if (!std::isfinite(v)) throw PimcError(kErrNonFinite, "non-finite bead coordinate");
                buf[((size_t)b * 3 + d) * np + g] = v;
            }
    if (which != 2) EnsureFP64();  // a partial update applies on top of the current state
    if (which == 0 || which == 2) CudaCheck(cudaMemcpyAsync(sys.pos, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice, stream), "set path");
    if (which == 1 || which == 2) CudaCheck(cudaMemcpyAsync(sys.pos_new, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice, stream), "set path");
    Sync();
    fp64_valid = true;
    if (which != 1) dd_valid = false;
    if (which == 2) {
        for (auto& a : actions) a.is_first_time = true;
        path_lost = false;
        InitRhoK();
    }
}

void Context::GetPath(int which, double* h) {
    EnsureFP64();
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    std::vector<double> buf((size_t)M * 3 * np);
    CudaCheck(cudaMemcpyAsync(buf.data(), which == 0 ? sys.pos : sys.pos_new, buf.size() * sizeof(double), cudaMemcpyDeviceToHost, stream), "get path");
    Sync();
    for (uint32_t g = 0; g < sys.n_total; ++g)
        for (uint32_t b = 0; b < M; ++b)
            for (uint32_t d = 0; d < n_d; ++d) h[((size_t)g * M + b) * n_d + d] = buf[((size_t)b * 3 + d) * np + g];
}

void Context::GetRhoK(uint32_t s, double* out) {
    if (s >= sys.S || sys.sp_rho[s] < 0 || !sys.rho_k) throw PimcError(kErrArg, "species keeps no charge density");
    EnsureFP64();
    const size_t n = (size_t)sys.M * sys.K;
    CudaCheck(cudaMemcpyAsync(out, sys.rho_k + (size_t)sys.sp_rho[s] * n, n * sizeof(double2), cudaMemcpyDeviceToHost, stream), "get rho_k");
    Sync();
}

void Context::GetKVecs(double* out) {
    for (uint32_t k = 0; k < sys.K; ++k)
        for (uint32_t d = 0; d < sys.n_d; ++d) out[(size_t)k * sys.n_d + d] = kint[k][d] * sys.box[d];
}

}  // namespace pimc
