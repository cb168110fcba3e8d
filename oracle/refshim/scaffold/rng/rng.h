// Reference build shim (test infrastructure): the `RNG` class simpimc's moves draw from (scaffold
// submodule, absent). Draws are scripted: the harness queues, per move attempt, the particle and
// first-bead indices (returned 1-based by UnifRand(n), as the reference subtracts one,
// bisect_class.h:40-41), one normal triple per resampled bead in the order the reference samples
// them (NormRand, bisect_class.h:90-91), and one uniform per level test (UnifRand(),
// bisect_class.h:114). The harness takes these from the oracle's counter-based stream, so the
// reference's moves see the same random numbers as the oracle's and the GPU's. Drawing from an
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
    void Clear() {
        ints_.clear();
        normals_.clear();
        unif_.clear();
    }
    size_t Pending() const { return ints_.size() + normals_.size() + unif_.size(); }

    uint32_t UnifRand(uint32_t) { return Pop(ints_); }
    uint32_t UnifRand(int) { return Pop(ints_); }
    double UnifRand() { return Pop(unif_); }
    double UnifRand(double a, double b) { return a + (b - a) * Pop(unif_); }
    void NormRand(scaffold::matrix::vec<double>& v, double mean, double sigma) {
        const std::vector<double> z = Pop(normals_);
        if (z.size() < v.size()) throw std::logic_error("RNG script: normal triple too short");
        for (size_t d = 0; d < v.size(); ++d) v(d) = mean + sigma * z[d];
    }

   private:
    int seed_;
    std::deque<uint32_t> ints_;
    std::deque<std::vector<double>> normals_;
    std::deque<double> unif_;
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
