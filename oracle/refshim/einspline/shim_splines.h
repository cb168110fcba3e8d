// Reference build shim (test infrastructure): the einspline entry points simpimc's headers call
// (call sites in free_spline_class.h and bare/ilkka/david_pair_action_class.h). einspline
// is fetched from an unpinned tarball at configure time and is not in the checkout, so its
// {NATURAL, NATURAL} interpolants are restated from their mathematical definition: the natural
// cubic spline through the data (second derivative zero at both ends), here in the first-derivative
// (slope) formulation, solved with a tridiagonal elimination and evaluated in Hermite form. The 2-D
// spline is the tensor product of natural splines: for a point (x, y) the splines along x of every
// grid row are evaluated at x and a natural spline along y through those values is evaluated at y.
// Arguments outside a 1-D grid are clamped to it; the 2-D spline continues its edge cells' cubics.
// Only these behaviours are the shim's choice; einspline's own out-of-grid behaviour is unknown.
#pragma once

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

typedef enum { PERIODIC, DERIV1, DERIV2, FLAT, NATURAL, ANTIPERIODIC } bc_code;

typedef struct {
    bc_code lCode, rCode;
    double lVal, rVal;
} BCtype_d;

typedef struct {
    double start, end;
    int num;
    double delta, delta_inv;
} Ugrid;

typedef struct {
    double start, end;
    double* points;
    int num_points;
} NUgrid;

namespace refshim {

/// Natural cubic spline through (x_i, y_i): node slopes k_i from the tridiagonal slope equations.
struct Natural1D {
    std::vector<double> x, y, k;

    void Build(const double* xs, const double* ys, int n) {
        x.assign(xs, xs + n);
        y.assign(ys, ys + n);
        k.assign(n, 0.);
        if (n < 2) return;
        std::vector<double> a(n, 0.), b(n, 0.), c(n, 0.), r(n, 0.);
        for (int i = 0; i < n; ++i) {
            if (i == 0) {
                const double h = x[1] - x[0];
                b[0] = 2. / h;
                c[0] = 1. / h;
                r[0] = 3. * (y[1] - y[0]) / (h * h);
            } else if (i == n - 1) {
                const double h = x[n - 1] - x[n - 2];
                a[i] = 1. / h;
                b[i] = 2. / h;
                r[i] = 3. * (y[n - 1] - y[n - 2]) / (h * h);
            } else {
                const double hl = x[i] - x[i - 1], hr = x[i + 1] - x[i];
                a[i] = 1. / hl;
                b[i] = 2. / hl + 2. / hr;
                c[i] = 1. / hr;
                r[i] = 3. * ((y[i] - y[i - 1]) / (hl * hl) + (y[i + 1] - y[i]) / (hr * hr));
            }
        }
        for (int i = 1; i < n; ++i) {  // forward elimination
            const double w = a[i] / b[i - 1];
            b[i] -= w * c[i - 1];
            r[i] -= w * r[i - 1];
        }
        k[n - 1] = r[n - 1] / b[n - 1];
        for (int i = n - 2; i >= 0; --i) k[i] = (r[i] - c[i] * k[i + 1]) / b[i];
    }

    int Cell(double t) const {
        const int n = (int)x.size();
        int i = (int)(std::upper_bound(x.begin(), x.end(), t) - x.begin()) - 1;
        return std::max(0, std::min(i, n - 2));
    }

    /// Value and derivative at t inside cell i (or its continuation past the grid ends).
    void CellVG(int i, double t, double& v, double& g) const {
        const double h = x[i + 1] - x[i];
        const double s = (t - x[i]) / h;
        const double s2 = s * s, s3 = s2 * s;
        const double h00 = 2. * s3 - 3. * s2 + 1., h10 = s3 - 2. * s2 + s, h01 = -2. * s3 + 3. * s2, h11 = s3 - s2;
        v = h00 * y[i] + h10 * h * k[i] + h01 * y[i + 1] + h11 * h * k[i + 1];
        const double d00 = 6. * s2 - 6. * s, d10 = 3. * s2 - 4. * s + 1., d01 = -6. * s2 + 6. * s, d11 = 3. * s2 - 2. * s;
        g = (d00 * y[i] + d01 * y[i + 1]) / h + d10 * k[i] + d11 * k[i + 1];
    }

    void EvalClampedVG(double t, double& v, double& g) const {
        t = std::min(std::max(t, x.front()), x.back());
        CellVG(Cell(t), t, v, g);
    }
    void EvalExtVG(double t, double& v, double& g) const { CellVG(Cell(t), t, v, g); }
};

}  // namespace refshim

struct UBspline_1d_d {
    refshim::Natural1D s;
};
struct NUBspline_1d_d {
    refshim::Natural1D s;
};
struct NUBspline_2d_d {
    std::vector<double> xg, yg;
    std::vector<refshim::Natural1D> rows;  // rows[j]: the spline along x of f(., y_j)
};
struct multi_NUBspline_1d_d {
    std::vector<double> grid;
    std::vector<refshim::Natural1D> comps;
};

inline UBspline_1d_d* create_UBspline_1d_d(Ugrid g, BCtype_d, double* data) {
    std::vector<double> xs(g.num);
    const double dx = (g.end - g.start) / (g.num - 1);
    for (int i = 0; i < g.num; ++i) xs[i] = g.start + i * dx;
    auto* s = new UBspline_1d_d();
    s->s.Build(xs.data(), data, g.num);
    return s;
}
inline void eval_UBspline_1d_d(UBspline_1d_d* s, double x, double* v) {
    double g;
    s->s.EvalClampedVG(x, *v, g);
}
inline void eval_UBspline_1d_d_vg(UBspline_1d_d* s, double x, double* v, double* g) { s->s.EvalClampedVG(x, *v, *g); }

inline NUgrid* create_general_grid(double* points, int n) {
    auto* g = new NUgrid();
    g->points = new double[n];
    std::copy(points, points + n, g->points);
    g->num_points = n;
    g->start = points[0];
    g->end = points[n - 1];
    return g;
}
inline NUgrid* create_linear_grid(double start, double end, int n) {
    std::vector<double> p(n);
    for (int i = 0; i < n; ++i) p[i] = start + (end - start) * i / (double)(n - 1);
    return create_general_grid(p.data(), n);
}
// The tables written by this repository use general grids; the other grid types are not restated.
inline NUgrid* create_log_grid(double, double, int) { throw std::runtime_error("reference build shim: LOG grids are not restated"); }
inline NUgrid* create_loglin_grid(double, double, double, int) { throw std::runtime_error("reference build shim: LOGLIN grids are not restated"); }

inline NUBspline_1d_d* create_NUBspline_1d_d(NUgrid* g, BCtype_d, double* data) {
    auto* s = new NUBspline_1d_d();
    s->s.Build(g->points, data, g->num_points);
    return s;
}
inline void eval_NUBspline_1d_d(NUBspline_1d_d* s, double x, double* v) {
    double g;
    s->s.EvalClampedVG(x, *v, g);
}
inline void eval_NUBspline_1d_d_vg(NUBspline_1d_d* s, double x, double* v, double* g) { s->s.EvalClampedVG(x, *v, *g); }

/// data[i n_y + j] = f(x_i, y_j).
inline NUBspline_2d_d* create_NUBspline_2d_d(NUgrid* xg, NUgrid* yg, BCtype_d, BCtype_d, double* data) {
    auto* s = new NUBspline_2d_d();
    const int nx = xg->num_points, ny = yg->num_points;
    s->xg.assign(xg->points, xg->points + nx);
    s->yg.assign(yg->points, yg->points + ny);
    s->rows.resize(ny);
    std::vector<double> col(nx);
    for (int j = 0; j < ny; ++j) {
        for (int i = 0; i < nx; ++i) col[i] = data[(size_t)i * ny + j];
        s->rows[j].Build(s->xg.data(), col.data(), nx);
    }
    return s;
}
inline void eval_NUBspline_2d_d_vg(NUBspline_2d_d* s, double x, double y, double* v, double* grad) {
    const int ny = (int)s->yg.size();
    std::vector<double> fv(ny), fx(ny);
    for (int j = 0; j < ny; ++j) s->rows[j].EvalExtVG(x, fv[j], fx[j]);
    refshim::Natural1D along_y, along_y_dx;
    along_y.Build(s->yg.data(), fv.data(), ny);
    along_y_dx.Build(s->yg.data(), fx.data(), ny);
    double gy, unused;
    along_y.EvalExtVG(y, *v, gy);
    along_y_dx.EvalExtVG(y, grad[0], unused);
    grad[1] = gy;
}
inline void eval_NUBspline_2d_d(NUBspline_2d_d* s, double x, double y, double* v) {
    double g[2];
    eval_NUBspline_2d_d_vg(s, x, y, v, g);
}

inline multi_NUBspline_1d_d* create_multi_NUBspline_1d_d(NUgrid* g, BCtype_d, int num_splines) {
    auto* s = new multi_NUBspline_1d_d();
    s->grid.assign(g->points, g->points + g->num_points);
    s->comps.resize(num_splines);
    return s;
}
inline void set_multi_NUBspline_1d_d(multi_NUBspline_1d_d* s, int i, double* data) {
    s->comps[i].Build(s->grid.data(), data, (int)s->grid.size());
}
inline void eval_multi_NUBspline_1d_d(multi_NUBspline_1d_d* s, double x, double* vals) {
    for (size_t i = 0; i < s->comps.size(); ++i) {
        double g;
        s->comps[i].EvalClampedVG(x, vals[i], g);
    }
}
inline void eval_multi_NUBspline_1d_d_vg(multi_NUBspline_1d_d* s, double x, double* vals, double* grads) {
    for (size_t i = 0; i < s->comps.size(); ++i) s->comps[i].EvalClampedVG(x, vals[i], grads[i]);
}
