// Reference build shim (test infrastructure): the `RNG` class simpimc's moves draw from (scaffold
// submodule, absent). Draws are scripted: the harness queues, per move attempt, the indices
// returned 1-based by UnifRand(n) in the order the move draws them (the reference subtracts one:
// Bisect's particle then first bead, bisect_class.h:40-41; the permuting moves' first bead then,
// for PermBisectIterative, the cycle's first particle, perm_bisect_iterative_class.h:114, 37), one
// normal triple per resampled bead in the order the reference samples them (NormRand,
// bisect_class.h:90-91), and the uniforms (UnifRand() and UnifRand(a, b)) in two queues: those a
// move draws before its first normal of the attempt (the permuting moves' cycle selection,
// perm_bisect_iterative_class.h:69-75, perm_bisect_table_class.h:106) and those it draws after it
// (every level test, bisect_class.h:114, and PermBisectTable's final test, :223). Splitting them
// lets the harness queue every selection uniform the attempt might need without knowing how many
// the cycle walk takes. The harness takes all of them from the oracle's counter-based stream, so
// the reference's moves see the same random numbers as the oracle's and the GPU's. Drawing from an
// empty queue is a harness error.
#pragma once

#include <cstdint>
#include <deque>
#include <stdexcept>
#include <vector>

#include "../matrix/matrix.h"

namespace scaffold {
namespace rand {

class RNG {
   public:
    explicit RNG(int seed = 0) : seed_(seed) {}
    void QueueIndex(uint32_t one_based) { ints_.push_back(one_based); }
    void QueueNormal(const std::vector<double>& z) { normals_.push_back(z); }
    void QueueUniform(double u) { unif_.push_back(u); }
    void QueueSelectionUniform(double u) { pre_.push_back(u); }
    void Clear() {
        ints_.clear();
        normals_.clear();
        unif_.clear();
        pre_.clear();
        sampled_ = false;
    }
    size_t Pending() const { return ints_.size() + normals_.size() + unif_.size() + pre_.size(); }

    uint32_t UnifRand(uint32_t) { return Pop(ints_); }
    uint32_t UnifRand(int) { return Pop(ints_); }
    double UnifRand() { return Pop(sampled_ ? unif_ : pre_); }
    double UnifRand(double a, double b) { return a + (b - a) * Pop(sampled_ ? unif_ : pre_); }
    void NormRand(scaffold::matrix::vec<double>& v, double mean, double sigma) {
        const std::vector<double> z = Pop(normals_);
        if (z.size() < v.size()) throw std::logic_error("RNG script: normal triple too short");
        for (size_t d = 0; d < v.size(); ++d) v(d) = mean + sigma * z[d];
        sampled_ = true;
    }

   private:
    int seed_;
    bool sampled_ = false;
    std::deque<uint32_t> ints_;
    std::deque<std::vector<double>> normals_;
    std::deque<double> unif_, pre_;
    template <class T>
    static T Pop(std::deque<T>& q) {
        if (q.empty()) throw std::logic_error("RNG script exhausted");
        T v = q.front();
        q.pop_front();
        return v;
    }
};

}  // namespace rand
}  // namespace scaffold
