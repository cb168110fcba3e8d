// Reference build shim (test infrastructure): the helper functions simpimc's headers take from the
// `scaffold` submodule, written from their call sites (the submodule is not in the checkout).
//   CMag2(a, b)   Re a Re b + Im a Im b (the structure factor uses it as |rho|^2,
//                 structure_factor_class.h:23);
//   fequal(a,b,t) |a - b| < t, the k-magnitude matching of the pair-action tables;
//   CompareVec    strict weak order of vectors (map keys of permutation sectors);
//   GenCombPermK  all k-tuples of the distinct values of a set, in lexicographic order. KSpace::Setup
//                 passes the concatenated index ranges of every dimension and k = n_d
//                 (k_space_class.h:59-64) and keeps each integer vector once; the scaffold order is
//                 unknown, so the tuples come in the order the oracle enumerates them.
#pragma once

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <vector>

namespace scaffold {
namespace algorithm {

inline double CMag2(const std::complex<double>& a, const std::complex<double>& b) { return a.real() * b.real() + a.imag() * b.imag(); }

inline bool fequal(double a, double b, double tol) { return std::fabs(a - b) < tol; }

template <class T>
struct CompareVec {
    bool operator()(const std::vector<T>& a, const std::vector<T>& b) const {
        return std::lexicographical_compare(a.begin(), a.end(), b.begin(), b.end());
    }
};

template <class T>
void GenCombPermK(std::vector<std::vector<T>>& out, const std::vector<T>& set, uint32_t k, bool /*unused*/, bool /*unused*/) {
    std::vector<T> vals(set);
    std::sort(vals.begin(), vals.end());
    vals.erase(std::unique(vals.begin(), vals.end()), vals.end());
    out.clear();
    if (k == 0 || vals.empty()) return;
    std::vector<size_t> idx(k, 0);
    for (;;) {
        std::vector<T> t(k);
        for (uint32_t i = 0; i < k; ++i) t[i] = vals[idx[i]];
        out.push_back(t);
        int d = (int)k - 1;
        while (d >= 0 && ++idx[d] == vals.size()) idx[d--] = 0;
        if (d < 0) break;
    }
}

}  // namespace algorithm
}  // namespace scaffold
