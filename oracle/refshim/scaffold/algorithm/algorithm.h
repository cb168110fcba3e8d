// Reference build shim (test infrastructure): the helper functions simpimc's headers take from the
// `scaffold` submodule, written from their call sites (the submodule is not in the checkout).
//   CMag2(a, b)   Re a Re b + Im a Im b (the structure factor uses it as |rho|^2,
//                 structure_factor_class.h:23);
//   fequal(a,b,t) |a - b| < t, the k-magnitude matching of the pair-action tables;
//   CompareVec    strict weak order of vectors (map keys of permutation sectors);
//   GenCombPermK  (set, k, repeat = false, ordered = true): all k-tuples of the distinct values of a
//                 set, in lexicographic order. KSpace::Setup passes the concatenated index ranges of
//                 every dimension and k = n_d (k_space_class.h:59-64) and keeps each integer vector
//                 once. (set, k, false, false): the k-element subsets of the set's elements, each
//                 in the set's order, subsets in lexicographic order of positions — the particle
//                 sets of PermBisectTable's cycles (perm_bisect_table_class.h:80-86). The scaffold
//                 orders are unknown, so both come in the order the oracle enumerates them.
//   GenPerm       every permutation of a vector, lexicographic from its given order (the
//                 permutation types of PermBisectTable, perm_bisect_table_class.h:55-61), the
//                 oracle's order.
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
void GenPerm(std::vector<std::vector<T>>& out, const std::vector<T>& v) {
    out.clear();
    std::vector<size_t> idx(v.size());
    for (size_t i = 0; i < idx.size(); ++i) idx[i] = i;
    do {
        std::vector<T> p(v.size());
        for (size_t i = 0; i < idx.size(); ++i) p[i] = v[idx[i]];
        out.push_back(p);
    } while (std::next_permutation(idx.begin(), idx.end()));
}

template <class T>
void GenCombPermK(std::vector<std::vector<T>>& out, const std::vector<T>& set, uint32_t k, bool repeat, bool ordered) {
    if (!repeat && !ordered) {  // subsets of k positions, lexicographic
        out.clear();
        const size_t n = set.size();
        if (k == 0 || k > n) return;
        std::vector<size_t> c(k);
        for (uint32_t i = 0; i < k; ++i) c[i] = i;
        for (;;) {
            std::vector<T> t(k);
            for (uint32_t i = 0; i < k; ++i) t[i] = set[c[i]];
            out.push_back(t);
            int i = (int)k - 1;
            while (i >= 0 && c[i] == n - k + (size_t)i) --i;
            if (i < 0) break;
            ++c[i];
            for (uint32_t j = (uint32_t)i + 1; j < k; ++j) c[j] = c[j - 1] + 1;
        }
        return;
    }
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
