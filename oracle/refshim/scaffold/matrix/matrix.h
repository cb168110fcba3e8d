// Reference build shim (test infrastructure): the dense-array surface simpimc's headers use from
// their `scaffold` submodule, which wraps Armadillo. Neither is part of the reference checkout, so
// this file provides the same names over std::vector, written from how the reference calls them:
// vec<T> (a column), mat<T> (column-major), cube<T> (column-major, then slices), field<T> (1-D or
// 2-D array of objects), zeros<>, dot, mag, sum and the element-wise arithmetic the headers use.
// Element storage is zero-initialised on construction and on set_size. Element access with () is
// bounds-checked and throws std::out_of_range, as Armadillo's is unless ARMA_NO_DEBUG is defined.
#pragma once

#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <initializer_list>
#include <iostream>
#include <stdexcept>
#include <type_traits>
#include <vector>

namespace scaffold {
namespace matrix {

template <class T>
class vec {
   public:
    typedef T elem_type;
    vec() = default;
    explicit vec(size_t n) : d_(n, T()) {}
    vec(std::initializer_list<T> l) : d_(l) {}

    size_t size() const { return d_.size(); }
    T* memptr() { return d_.data(); }
    const T* memptr() const { return d_.data(); }
    T& operator()(size_t i) { return d_.at(i); }
    const T& operator()(size_t i) const { return d_.at(i); }
    T& operator[](size_t i) { return d_[i]; }
    const T& operator[](size_t i) const { return d_[i]; }
    void set_size(size_t n) { d_.assign(n, T()); }
    void resize(size_t n) { d_.resize(n, T()); }
    vec& zeros() {
        for (auto& x : d_) x = T();
        return *this;
    }
    vec& zeros(size_t n) {
        d_.assign(n, T());
        return *this;
    }
    void fill(const T& v) {
        for (auto& x : d_) x = v;
    }
    typename std::vector<T>::iterator begin() { return d_.begin(); }
    typename std::vector<T>::iterator end() { return d_.end(); }
    typename std::vector<T>::const_iterator begin() const { return d_.begin(); }
    typename std::vector<T>::const_iterator end() const { return d_.end(); }

    vec& operator+=(const vec& o) {
        Check(o);
        for (size_t i = 0; i < d_.size(); ++i) d_[i] += o.d_[i];
        return *this;
    }
    vec& operator-=(const vec& o) {
        Check(o);
        for (size_t i = 0; i < d_.size(); ++i) d_[i] -= o.d_[i];
        return *this;
    }
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    vec& operator*=(S s) {
        for (auto& x : d_) x *= s;
        return *this;
    }
    template <class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
    vec& operator/=(S s) {
        for (auto& x : d_) x /= s;
        return *this;
    }

   private:
    std::vector<T> d_;
    void Check(const vec& o) const {
        if (o.d_.size() != d_.size()) throw std::logic_error("vec: size mismatch");
    }
};

template <class T>
vec<T> operator+(const vec<T>& a, const vec<T>& b) {
    vec<T> r(a);
    r += b;
    return r;
}
template <class T>
vec<T> operator-(const vec<T>& a, const vec<T>& b) {
    vec<T> r(a);
    r -= b;
    return r;
}
template <class T>
vec<T> operator-(const vec<T>& a) {
    vec<T> r(a.size());
    for (size_t i = 0; i < a.size(); ++i) r(i) = -a(i);
    return r;
}
template <class T, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
vec<T> operator*(const vec<T>& a, S s) {
    vec<T> r(a);
    r *= s;
    return r;
}
template <class T, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
vec<T> operator*(S s, const vec<T>& a) {
    vec<T> r(a.size());
    for (size_t i = 0; i < a.size(); ++i) r(i) = s * a(i);
    return r;
}
template <class T, class S, class = typename std::enable_if<std::is_arithmetic<S>::value>::type>
vec<T> operator/(const vec<T>& a, S s) {
    vec<T> r(a);
    r /= s;
    return r;
}
template <class T>
std::ostream& operator<<(std::ostream& o, const vec<T>& v) {
    for (size_t i = 0; i < v.size(); ++i) o << v(i) << (i + 1 < v.size() ? " " : "");
    return o;
}

template <class T>
T dot(const vec<T>& a, const vec<T>& b) {
    T t = T();
    for (size_t i = 0; i < a.size(); ++i) t += a(i) * b(i);
    return t;
}
template <class T>
double mag(const vec<T>& a) {
    return std::sqrt(dot(a, a));
}
template <class T>
double Mag(const vec<T>& a) {
    return mag(a);
}
template <class T>
T sum(const vec<T>& a) {
    T t = T();
    for (const auto& x : a) t += x;
    return t;
}

template <class T>
class mat {
   public:
    typedef T elem_type;
    size_t n_rows = 0, n_cols = 0;
    mat() = default;
    mat(size_t r, size_t c) : n_rows(r), n_cols(c), d_(r * c, T()) {}
    size_t size() const { return d_.size(); }
    T* memptr() { return d_.data(); }
    const T* memptr() const { return d_.data(); }
    T& operator()(size_t i, size_t j) { return d_.at(Idx(i, j)); }
    const T& operator()(size_t i, size_t j) const { return d_.at(Idx(i, j)); }
    T& operator()(size_t i) { return d_.at(i); }
    const T& operator()(size_t i) const { return d_.at(i); }
    void set_size(size_t r, size_t c) {
        n_rows = r;
        n_cols = c;
        d_.assign(r * c, T());
    }
    mat& zeros() {
        for (auto& x : d_) x = T();
        return *this;
    }
    mat& zeros(size_t r, size_t c) {
        set_size(r, c);
        return *this;
    }

   private:
    std::vector<T> d_;
    size_t Idx(size_t i, size_t j) const {
        if (i >= n_rows || j >= n_cols) throw std::out_of_range("mat index");
        return i + j * n_rows;
    }
};

template <class T>
class cube {
   public:
    typedef T elem_type;
    size_t n_rows = 0, n_cols = 0, n_slices = 0;
    cube() = default;
    cube(size_t r, size_t c, size_t s) : n_rows(r), n_cols(c), n_slices(s), d_(r * c * s, T()) {}
    size_t size() const { return d_.size(); }
    T* memptr() { return d_.data(); }
    const T* memptr() const { return d_.data(); }
    T& operator()(size_t i, size_t j, size_t k) { return d_.at(Idx(i, j, k)); }
    const T& operator()(size_t i, size_t j, size_t k) const { return d_.at(Idx(i, j, k)); }
    void set_size(size_t r, size_t c, size_t s) {
        n_rows = r;
        n_cols = c;
        n_slices = s;
        d_.assign(r * c * s, T());
    }
    cube& zeros() {
        for (auto& x : d_) x = T();
        return *this;
    }

   private:
    std::vector<T> d_;
    size_t Idx(size_t i, size_t j, size_t k) const {
        if (i >= n_rows || j >= n_cols || k >= n_slices) throw std::out_of_range("cube index");
        return i + n_rows * (j + n_cols * k);
    }
};

/// A 1-D or 2-D (column-major) array of arbitrary objects.
template <class T>
class field {
   public:
    size_t n_rows = 0, n_cols = 0;
    field() = default;
    explicit field(size_t n) : n_rows(n), n_cols(1), d_(n) {}
    field(size_t r, size_t c) : n_rows(r), n_cols(c), d_(r * c) {}
    size_t size() const { return d_.size(); }
    T& operator()(size_t i) { return d_.at(i); }
    const T& operator()(size_t i) const { return d_.at(i); }
    T& operator()(size_t i, size_t j) {
        if (i >= n_rows || j >= n_cols) throw std::out_of_range("field index");
        return d_[i + j * n_rows];
    }
    const T& operator()(size_t i, size_t j) const {
        if (i >= n_rows || j >= n_cols) throw std::out_of_range("field index");
        return d_[i + j * n_rows];
    }
    void set_size(size_t n) {
        n_rows = n;
        n_cols = 1;
        d_.assign(n, T());
    }
    void set_size(size_t r, size_t c) {
        n_rows = r;
        n_cols = c;
        d_.assign(r * c, T());
    }
    typename std::vector<T>::iterator begin() { return d_.begin(); }
    typename std::vector<T>::iterator end() { return d_.end(); }

   private:
    std::vector<T> d_;
};

/// Matrix-vector product (PermBisectTable forms inverse permutations as a permutation matrix times
/// an index vector, perm_bisect_table_class.h:67-77).
template <class T>
vec<T> operator*(const mat<T>& m, const vec<T>& v) {
    if (m.n_cols != v.size()) throw std::logic_error("mat * vec: size mismatch");
    vec<T> r(m.n_rows);
    for (size_t i = 0; i < m.n_rows; ++i) {
        T t = T();
        for (size_t j = 0; j < m.n_cols; ++j) t += m(i, j) * v(j);
        r(i) = t;
    }
    return r;
}

template <class V>
V zeros(size_t n) {
    return V(n);
}
template <class V>
V zeros(size_t r, size_t c) {
    return V(r, c);
}

}  // namespace matrix
}  // namespace scaffold
