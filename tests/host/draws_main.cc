// Host build of the product's random-number header: prints the draws of one bisection attempt
// (the same quantities as oracle_bisect_draws) for the CPU test of the transforms' bit identity.
#include <cstdio>
#include <cstdlib>

#include "../../simpimc_gb300/src/common/philox.h"

int main(int argc, char** argv) {
    if (argc != 8) return 2;
    const uint32_t seed = (uint32_t)strtoul(argv[1], nullptr, 10), chain = (uint32_t)strtoul(argv[2], nullptr, 10);
    const uint32_t move = (uint32_t)strtoul(argv[3], nullptr, 10);
    const uint64_t attempt = strtoull(argv[4], nullptr, 10);
    const uint32_t n_part = (uint32_t)strtoul(argv[5], nullptr, 10), n_bead = (uint32_t)strtoul(argv[6], nullptr, 10);
    const uint32_t n_level = (uint32_t)strtoul(argv[7], nullptr, 10);
    const pimc::MoveStream st{seed, chain, move, attempt};
    const pimc::Philox4 w0 = st.Block(0);
    printf("%u %u\n", pimc::UniformIndex(w0.v[0], n_part), pimc::UniformIndex(w0.v[1], n_bead));
    const uint32_t B = 1u << n_level;
    for (uint32_t i = 0; i + 1 < B; ++i) {
        float z[3];
        pimc::BisectNormals(st, i, z);
        printf("%08x %08x %08x\n", pimc::FloatBits(z[0]), pimc::FloatBits(z[1]), pimc::FloatBits(z[2]));
    }
    for (uint32_t li = 0; li < n_level; ++li) printf("%08x\n", pimc::FloatBits(pimc::BisectLogU(st, B, li)));
    return 0;
}
