// pimc_get_action_noalloc: the pair-action GetAction with no device allocation inside the call.
//
// Why it exists: some host programs hand (nearly) all GPU memory to their own allocator or pool
// when they start, so a cudaMalloc issued later by a library either fails or goes behind the
// pool's accounting; others call into this library from code where a device allocation is not
// allowed at all. pimc_get_action may grow its per-context scratch buffers with cudaMalloc when
// a request is larger than every earlier one. This entry point computes the same value but keeps
// every temporary (pair list, particle lists, the proposal's charge densities, the reduction
// partials and the result slot) in one fixed device array declared in this file.
//
// The array is kNoAllocScratchBytes = 4 MiB. CUDA loads a module's device variables and kernels
// lazily by default, so pimc_create calls NoAllocPrepare: it looks up the array's address (which
// loads this file's module and so places the array on the GPU) and loads every kernel the entry
// point launches, including the FP64 conversion kernels of the sweep. From then on the GPU holds
// the array until the process exits, and a call allocates nothing. A request needs, each part
// rounded up to 256 bytes: 8 bytes per particle pair, 4 bytes per listed particle, 16 bytes per
// (slice, k-vector) and species for NEW-mode long-range actions, and 8 bytes per reduction block
// plus 64 bytes; anything larger is refused with PIMC_ERR_ARG and a message stating the need.
//
// All calls share the array and it keeps whatever the last call left in it. Nothing in it has to
// start at zero: every region is fully written before it is read. Two calls whose GPU work
// overlaps (for example from two contexts on one device, driven by different host threads) race
// on the array; calls on one context are serialised by its stream and by the synchronisation at
// the end of each call.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/simpimc_gb300.h"
#include "capi_internal.h"
#include "kernels/actions.cuh"

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr int kNoAllocMaxDevices = 64;
constexpr int kNoAllocThreads = 256;

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {

std::mutex g_noalloc_mu;
void* g_noalloc_addr[kNoAllocMaxDevices] = {nullptr};

/// Device address of the scratch array on `device` (looked up once per device).
void* ScratchAddress(int device) {
    if (device < 0 || device >= kNoAllocMaxDevices) throw pimc::PimcError(PIMC_ERR_ARG, "device ordinal out of range for the scratch table");
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_addr[device]) {
        int prev = 0;
        pimc::CudaCheck(cudaGetDevice(&prev), "cudaGetDevice");
        pimc::CudaCheck(cudaSetDevice(device), "cudaSetDevice");
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        cudaSetDevice(prev);
        pimc::CudaCheck(e, "cudaGetSymbolAddress(scratch)");
        g_noalloc_addr[device] = p;
    }
    return g_noalloc_addr[device];
}

size_t Round256(size_t n) { return (n + 255) & ~size_t(255); }

__device__ __forceinline__ uint32_t Loop(uint32_t b, uint32_t M) { return b >= M ? b - M : b; }

template <class F>
__global__ void __launch_bounds__(kNoAllocThreads) NoAllocSumKernel(uint64_t n, F f, double* __restrict__ partials) {
    __shared__ double red[kNoAllocThreads / 32];
    double acc = 0.;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) acc += f(i);
    const double s = pimc::BlockSum(acc, red);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void NoAllocFinalKernel(const double* __restrict__ partials, int nb, double* __restrict__ out) {
    double t = 0.;
    for (int b = threadIdx.x; b < nb; b += 32) t += partials[b];
    t = pimc::WarpSum(t);
    if (threadIdx.x == 0) *out = t;
}

// Proposal densities of one species on the segment: committed density plus (new - old) phases of
// the listed particles in list order (species_class.h:406-425).
__global__ void NoAllocProposalRhoKernel(const pimc::SystemDev sys, uint32_t species, const uint32_t* __restrict__ parts,
                                         uint32_t n_parts, uint32_t b0, uint32_t skip, double2* __restrict__ out) {
    extern __shared__ double2 tab[];
    const uint32_t j = blockIdx.x;
    const uint32_t b = Loop(b0 + j * skip, sys.M);
    const int stride = max(max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
    const double2* committed = sys.rho_k + ((size_t)sys.sp_rho[species] * sys.M + b) * sys.K;
    double2* dst = out + (size_t)j * sys.K;
    for (uint32_t k = threadIdx.x; k < sys.K; k += blockDim.x) dst[k] = committed[k];
    for (uint32_t q = 0; q < n_parts; ++q) {
        const uint32_t g = sys.sp_off[species] + parts[q];
        __syncthreads();
        if (threadIdx.x < 2 * sys.n_d) {
            const uint32_t which = threadIdx.x / sys.n_d, d = threadIdx.x % sys.n_d;
            const double x = pimc::PosAt(which ? sys.pos_new : sys.pos, sys.n_pad, b, d, g);
            pimc::PhaseRow(x, sys.box[d], sys.max_index[d], tab + ((size_t)which * 3 + d) * stride);
        }
        __syncthreads();
        for (uint32_t k = threadIdx.x; k < sys.K; k += blockDim.x) {
            const int32_t pk = sys.kidx[k];
            const double2 en = pimc::PhaseProduct(tab + (size_t)3 * stride, stride, sys.n_d, pk);
            const double2 eo = pimc::PhaseProduct(tab, stride, sys.n_d, pk);
            double2 v = dst[k];
            v.x += en.x - eo.x;
            v.y += en.y - eo.y;
            dst[k] = v;
        }
    }
}

// One (slice, pair) link of PairAction::GetAction (pair_action_class.h:278-289).
struct NoAllocPairTerm {
    pimc::PairDev pa;
    const double* pos;
    const uint32_t* pairs;
    uint32_t npairs, b0, skip, M, n_d, np, offa, offb, level;
    double L, iL, tau;
    __device__ double operator()(uint64_t i) const {
        const uint32_t j = (uint32_t)(i / npairs), q = (uint32_t)(i % npairs);
        const uint32_t bi = Loop(b0 + j * skip, M), bj = Loop(b0 + j * skip + skip, M);
        double A0[3], C0[3], A1[3], C1[3];
        pimc::LoadBead(pos, np, n_d, bi, offb + pairs[2 * q + 1], A0);
        pimc::LoadBead(pos, np, n_d, bi, offa + pairs[2 * q], C0);
        pimc::LoadBead(pos, np, n_d, bj, offb + pairs[2 * q + 1], A1);
        pimc::LoadBead(pos, np, n_d, bj, offa + pairs[2 * q], C1);
        double r, rp, s;
        pimc::DrDrpDrrp(A0, C0, A1, C1, n_d, L, iL, r, rp, s);
        return pimc::PairU(pa, r, rp, s, level, tau);
    }
};

// One (k-vector, slice) term of the long-range sum v_k Re(rho_a conj(rho_b)) (bare_pair_action_class.h:
// 126-144): from the proposal densities `ra`/`rb` (NEW mode) or the committed per-slice densities.
struct NoAllocLongTerm {
    const double2* ra;
    const double2* rb;
    const double2* rho;
    const double* vk;
    uint32_t K, ns, b0, skip, M;
    int slot_a, slot_b;
    __device__ double operator()(uint64_t i) const {
        const uint32_t k = (uint32_t)(i / ns), j = (uint32_t)(i % ns);
        double2 a, b;
        if (ra) {
            a = ra[(size_t)j * K + k];
            b = rb[(size_t)j * K + k];
        } else {
            const uint32_t bb = Loop(b0 + j * skip, M);
            a = rho[((size_t)slot_a * M + bb) * K + k];
            b = rho[((size_t)slot_b * M + bb) * K + k];
        }
        return vk[k] * (a.x * b.x + a.y * b.y);
    }
};

/// Sum f over [0, n) into *result using `partials` (capacity `cap` doubles) in the scratch array.
template <class F>
double NoAllocSum(pimc::Context& c, uint64_t n, F f, double* partials, size_t cap, double* result) {
    if (n == 0) return 0.;
    const uint64_t want = (n + kNoAllocThreads - 1) / kNoAllocThreads;
    const int blocks = (int)std::max<uint64_t>(1, std::min<uint64_t>({want, (uint64_t)c.n_sm * 8, (uint64_t)cap}));
    NoAllocSumKernel<<<blocks, kNoAllocThreads, 0, c.stream>>>(n, f, partials);
    pimc::CudaCheck(cudaGetLastError(), "no-alloc sum launch");
    NoAllocFinalKernel<<<1, 32, 0, c.stream>>>(partials, blocks, result);
    pimc::CudaCheck(cudaGetLastError(), "no-alloc final launch");
    double h = 0.;
    pimc::CudaCheck(cudaMemcpyAsync(&h, result, sizeof(double), cudaMemcpyDeviceToHost, c.stream), "no-alloc result");
    c.Sync();
    return h;
}

double GetActionNoAlloc(pimc::Context& c, uint32_t ai, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n,
                        uint32_t level, int mode) {
    using pimc::PimcError;
    if (ai >= c.actions.size()) throw PimcError(PIMC_ERR_ARG, "action index out of range");
    if (level >= (uint32_t)pimc::kMaxLevels) throw PimcError(PIMC_ERR_ARG, "level out of range");
    if (b1 < b0 || b0 >= c.sys.M || b1 - b0 > c.sys.M) throw PimcError(PIMC_ERR_ARG, "slice range out of bounds");
    const pimc::ActionHost& ah = c.actions[ai];
    if (ah.kind != 2) throw PimcError(PIMC_ERR_UNSUPPORTED, "pimc_get_action_noalloc evaluates pair actions only");
    c.EnsureFP64();  // a conversion kernel when a sweep ran since the last FP64 read; no allocation
    const pimc::SystemDev& sys = c.sys;
    const pimc::PairDev pa = sys.pair[ah.index];
    if (level > pa.max_level || pa.is_constant) return 0.;

    // PairAction::GenerateParticlePairs (pair_action_class.h:62-114).
    std::vector<uint32_t> la, lb, pairs;
    for (uint32_t i = 0; i < n; ++i) {
        if (sp[i] >= sys.S || p[i] >= sys.sp_n[sp[i]]) throw PimcError(PIMC_ERR_ARG, "particle out of range");
        if (sp[i] == pa.sa) la.push_back(p[i]);
        else if (sp[i] == pa.sb) lb.push_back(p[i]);
    }
    if (la.empty() && lb.empty()) return 0.;
    std::vector<uint32_t> oa, ob;
    for (uint32_t i = 0; i < sys.sp_n[pa.sa]; ++i)
        if (std::find(la.begin(), la.end(), i) == la.end()) oa.push_back(i);
    for (uint32_t i = 0; i < sys.sp_n[pa.sb]; ++i)
        if (std::find(lb.begin(), lb.end(), i) == lb.end()) ob.push_back(i);
    auto add = [&](uint32_t x, uint32_t y) {
        pairs.push_back(x);
        pairs.push_back(y);
    };
    if (pa.sa == pa.sb) {
        for (auto x : la)
            for (auto y : oa) add(x, y);
        for (size_t i = 0; i + 1 < la.size(); ++i)
            for (size_t j = i + 1; j < la.size(); ++j) add(la[i], la[j]);
    } else {
        for (auto x : la)
            for (auto y : ob) add(x, y);
        for (auto x : lb)
            for (auto y : oa) add(y, x);
        for (auto x : la)
            for (auto y : lb) add(x, y);
    }
    const uint32_t npairs = (uint32_t)(pairs.size() / 2);
    if (npairs == 0) return 0.;
    const uint32_t skip = 1u << level;
    const uint32_t ns = (b1 - b0 + skip - 1) / skip;
    // The last link's far slice, b0 + ns skip, must lie within one wrap of the ring: the reference's
    // bead_loop subtracts M once (species_class.h:101), so beyond that it reads past its bead array.
    if ((uint64_t)b0 + (uint64_t)ns * skip >= 2ull * sys.M)
        throw PimcError(PIMC_ERR_ARG, "slice range reaches past one wrap of the ring at this level");
    const bool lr_new = pa.use_long_range && mode;
    const int n_species = pa.sa == pa.sb ? 1 : 2;

    // Scratch layout and size check.
    const size_t max_blocks = (size_t)c.n_sm * 8;
    const size_t off_pairs = 0;
    const size_t off_parts = off_pairs + Round256(pairs.size() * sizeof(uint32_t));
    const size_t off_rho = off_parts + Round256((la.size() + lb.size()) * sizeof(uint32_t));
    const size_t rho_bytes = lr_new ? (size_t)n_species * ns * sys.K * sizeof(double2) : 0;
    const size_t off_part = off_rho + Round256(rho_bytes);
    const size_t off_res = off_part + Round256(max_blocks * sizeof(double));
    const size_t need = off_res + 64;
    if (need > kNoAllocScratchBytes)
        throw PimcError(PIMC_ERR_ARG, "request needs " + std::to_string(need) + " bytes of scratch; the no-allocation limit is " +
                                          std::to_string(kNoAllocScratchBytes) + " bytes (use pimc_get_action)");

    pimc::CudaCheck(cudaSetDevice(c.device), "cudaSetDevice");
    unsigned char* base = static_cast<unsigned char*>(ScratchAddress(c.device));
    uint32_t* dp = reinterpret_cast<uint32_t*>(base + off_pairs);
    uint32_t* dl = reinterpret_cast<uint32_t*>(base + off_parts);
    double2* tmp = reinterpret_cast<double2*>(base + off_rho);
    double* partials = reinterpret_cast<double*>(base + off_part);
    double* result = reinterpret_cast<double*>(base + off_res);

    pimc::CudaCheck(cudaMemcpyAsync(dp, pairs.data(), pairs.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream), "pairs upload");
    std::vector<uint32_t> lists = la;
    lists.insert(lists.end(), lb.begin(), lb.end());
    if (!lists.empty())
        pimc::CudaCheck(cudaMemcpyAsync(dl, lists.data(), lists.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, c.stream), "parts upload");

    const double* pos = mode ? sys.pos_new : sys.pos;
    const uint32_t M = sys.M, n_d = sys.n_d, np = sys.n_pad;
    const double L = sys.L, iL = sys.iL, tau = sys.tau;
    const uint32_t offa = sys.sp_off[pa.sa], offb = sys.sp_off[pa.sb];
    NoAllocPairTerm pt;
    pt.pa = pa;
    pt.pos = pos;
    pt.pairs = dp;
    pt.npairs = npairs;
    pt.b0 = b0;
    pt.skip = skip;
    pt.M = M;
    pt.n_d = n_d;
    pt.np = np;
    pt.offa = offa;
    pt.offb = offb;
    pt.level = level;
    pt.L = L;
    pt.iL = iL;
    pt.tau = tau;
    double tot = NoAllocSum(c, (uint64_t)ns * npairs, pt, partials, max_blocks, result);

    if (pa.use_long_range) {
        const uint32_t K = sys.K;
        const int stride = std::max(std::max(sys.max_index[0], sys.max_index[1]), sys.max_index[2]) + 1;
        const double2* ra = nullptr;
        const double2* rb = nullptr;
        if (mode) {
            const uint32_t spc[2] = {pa.sa, pa.sb};
            const uint32_t* lptr[2] = {dl, dl + la.size()};
            const uint32_t lcnt[2] = {(uint32_t)la.size(), (uint32_t)lb.size()};
            for (int x = 0; x < n_species; ++x) {
                NoAllocProposalRhoKernel<<<ns, 256, (size_t)2 * 3 * stride * sizeof(double2), c.stream>>>(
                    sys, spc[x], lptr[x], lcnt[x], b0, skip, tmp + (size_t)x * ns * K);
                pimc::CudaCheck(cudaGetLastError(), "no-alloc proposal launch");
            }
            ra = tmp;
            rb = n_species == 1 ? tmp : tmp + (size_t)ns * K;
        }
        NoAllocLongTerm lt;
        lt.ra = ra;
        lt.rb = rb;
        lt.rho = sys.rho_k;
        lt.vk = pa.kind != pimc::kPairBare ? pa.u_long_k : pa.v_long_k;
        lt.K = K;
        lt.ns = ns;
        lt.b0 = b0;
        lt.skip = skip;
        lt.M = M;
        lt.slot_a = sys.sp_rho[pa.sa];
        lt.slot_b = sys.sp_rho[pa.sb];
        double lr = NoAllocSum(c, (uint64_t)K * ns, lt, partials, max_blocks, result);
        if (pa.sa != pa.sb) lr *= 2.;
        tot += pa.kind != pimc::kPairBare ? lr : skip * sys.tau * lr;
    }
    return tot;
}

}  // namespace

namespace pimc {

void NoAllocPrepare(int device) {
    static bool prepared[kNoAllocMaxDevices] = {false};
    ScratchAddress(device);  // loads this file's module: the scratch array is placed on the GPU here
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (prepared[device]) return;
    int prev = 0;
    CudaCheck(cudaGetDevice(&prev), "cudaGetDevice");
    CudaCheck(cudaSetDevice(device), "cudaSetDevice");
    // cudaFuncGetAttributes loads a kernel that lazy loading would otherwise load at its first launch.
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, NoAllocSumKernel<NoAllocPairTerm>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, NoAllocSumKernel<NoAllocLongTerm>);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, NoAllocFinalKernel);
    if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, NoAllocProposalRhoKernel);
    if (e == cudaSuccess) {
        try {
            PreloadConversionKernels();
        } catch (...) {
            cudaSetDevice(prev);
            throw;
        }
    }
    cudaSetDevice(prev);
    CudaCheck(e, "loading the no-allocation kernels");
    prepared[device] = true;
}

}  // namespace pimc

extern "C" int pimc_get_action_noalloc(pimc_ctx* ctx, uint32_t action, uint32_t b0, uint32_t b1, const uint32_t* species,
                                       const uint32_t* particles, uint32_t n_particles, uint32_t level, int mode, double* out) {
    if (!ctx || !ctx->c || !out || (n_particles && (!species || !particles))) return PIMC_ERR_ARG;
    try {
        *out = GetActionNoAlloc(*ctx->c, action, b0, b1, species, particles, n_particles, level, mode);
        return PIMC_OK;
    } catch (const pimc::PimcError& e) {
        ctx->err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        ctx->err = e.what();
        return PIMC_ERR_STATE;
    }
}
