// Host side of exchanging paths: the path permutation at the ring closure (bead (g, M - 1) is
// followed by bead (perm[g], 0), the representation the reference's bead links take after the
// relabelling of perm_bisect_class.h:47-56), its cycles and sign (species_class.h:28-45, 149-157),
// and which species need the permutation kernel. The kernel itself (double-float) is
// perm_dd.cuh, compiled with the sweep kernel's descriptors in sweep.cu.
#include <vector>

#include "../framework/context.h"

namespace pimc {

void Context::SyncPermHost() {
    if (perm_host.size() != sys.n_total) perm_host.resize(sys.n_total);
    CudaCheck(cudaMemcpyAsync(perm_host.data(), perm_->ptr, sys.n_total * sizeof(uint32_t), cudaMemcpyDeviceToHost, stream), "read perm");
    Sync();
}

bool Context::PermIdentity(uint32_t s) const {
    for (uint32_t p = 0; p < sys.sp_n[s]; ++p)
        if (perm_host[sys.sp_off[s] + p] != sys.sp_off[s] + p) return false;
    return true;
}

bool Context::AnyPerm() const {
    for (uint32_t s = 0; s < sys.S; ++s)
        if (!PermIdentity(s)) return true;
    return false;
}

void Context::SetPerm(uint32_t s, const uint32_t* pi) {
    if (s >= sys.S) throw PimcError(kErrArg, "species index out of range");
    const uint32_t N = sys.sp_n[s], G0 = sys.sp_off[s];
    std::vector<char> seen(N, 0);
    for (uint32_t p = 0; p < N; ++p) {
        if (pi[p] >= N || seen[pi[p]]) throw PimcError(kErrArg, "not a permutation of the species' particles");
        seen[pi[p]] = 1;
    }
    for (uint32_t p = 0; p < N; ++p) perm_host[G0 + p] = G0 + pi[p];
    std::vector<uint32_t> inv(sys.n_total);
    for (uint32_t g = 0; g < sys.n_total; ++g) inv[perm_host[g]] = g;
    CudaCheck(cudaMemcpyAsync(perm_->ptr, perm_host.data(), sys.n_total * sizeof(uint32_t), cudaMemcpyHostToDevice, stream), "write perm");
    CudaCheck(cudaMemcpyAsync(perm_inv_->ptr, inv.data(), sys.n_total * sizeof(uint32_t), cudaMemcpyHostToDevice, stream), "write perm");
    Sync();
}

void Context::GetPerm(uint32_t s, uint32_t* out) const {
    if (s >= sys.S) throw PimcError(kErrArg, "species index out of range");
    for (uint32_t p = 0; p < sys.sp_n[s]; ++p) out[p] = perm_host[sys.sp_off[s] + p] - sys.sp_off[s];
}

double Context::PathSign() const {
    // Path::GetSign (path_class.h:169-175): (-1)^(length - 1) per cycle of every fermion species
    int sign = 1;
    for (uint32_t s = 0; s < sys.S; ++s) {
        if (!species_fermi[s]) continue;
        for (uint32_t len : CycleLengths(s))
            if (!(len % 2)) sign = -sign;
    }
    return (double)sign;
}

std::vector<uint32_t> Context::CycleLengths(uint32_t s) const {
    // Species::SetCycleCount (species_class.h:28-45)
    const uint32_t N = sys.sp_n[s], G0 = sys.sp_off[s];
    std::vector<char> seen(N, 0);
    std::vector<uint32_t> out;
    for (uint32_t p = 0; p < N; ++p) {
        if (seen[p]) continue;
        uint32_t len = 0, q = p;
        do {
            seen[q] = 1;
            q = perm_host[G0 + q] - G0;
            ++len;
        } while (q != p && len <= N);
        out.push_back(len);
    }
    return out;
}

bool Context::PermutingSpecies(uint32_t s) const {
    for (const auto& mh : moves)
        if ((mh.kind == 2 || mh.kind == 3) && mh.dev.species == s) return true;
    return !PermIdentity(s);
}

}  // namespace pimc
