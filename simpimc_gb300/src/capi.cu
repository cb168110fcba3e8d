// C interface (include/simpimc_gb300.h) over pimc::Context. Exceptions never cross the boundary:
// each entry point converts them into a status code and keeps the message on the context.
#include <cstring>
#include <string>
#include <vector>

#include "../../include/simpimc_gb300.h"

#include "capi_internal.h"

namespace {

thread_local std::string g_create_error;

template <class F>
int Guard(pimc_ctx* ctx, F f) {
    if (!ctx || !ctx->c) return PIMC_ERR_ARG;
    try {
        f(*ctx->c);
        return PIMC_OK;
    } catch (const pimc::PimcError& e) {
        ctx->err = e.what();
        return e.code;
    } catch (const pimc::InputError& e) {
        ctx->err = e.what();
        return PIMC_ERR_INPUT;
    } catch (const std::exception& e) {
        ctx->err = e.what();
        return PIMC_ERR_STATE;
    }
}

}  // namespace

extern "C" {

int pimc_create(const char* xml_text, const char* base_dir, int device, uint32_t chain, pimc_ctx** out) {
    if (!xml_text || !out) return PIMC_ERR_ARG;
    *out = nullptr;
    try {
        pimc::Input in = pimc::Input::FromString(xml_text);
        std::unique_ptr<pimc_ctx> h(new pimc_ctx());
        h->c.reset(new pimc::Context(in, base_dir ? base_dir : "", device, chain));
        pimc::NoAllocPrepare(device);
        *out = h.release();
        return PIMC_OK;
    } catch (const pimc::PimcError& e) {
        g_create_error = e.what();
        return e.code;
    } catch (const pimc::InputError& e) {
        g_create_error = e.what();
        return PIMC_ERR_INPUT;
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return PIMC_ERR_STATE;
    }
}

void pimc_destroy(pimc_ctx* ctx) { delete ctx; }

const char* pimc_last_error(const pimc_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

int pimc_get_info(pimc_ctx* ctx, pimc_info* out) {
    if (!out) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        out->n_d = c.sys.n_d;
        out->n_bead = c.sys.M;
        out->n_species = c.sys.S;
        out->n_total = c.sys.n_total;
        out->n_k = c.sys.K;
        out->n_actions = (uint32_t)c.actions.size();
        out->n_moves = (uint32_t)c.moves.size();
        out->n_observables = (uint32_t)c.observables.size();
        out->beta = c.sys.beta;
        out->tau = c.sys.tau;
        out->L = c.sys.L;
        out->volume = c.sys.vol;
        out->pbc = c.sys.pbc;
    });
}

int pimc_set_seed(pimc_ctx* ctx, uint32_t seed) {
    return Guard(ctx, [&](pimc::Context& c) { c.seed = seed; });
}

int pimc_get_name(pimc_ctx* ctx, int kind, uint32_t index, char* buf, size_t cap) {
    if (!buf || cap == 0) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        std::string s;
        if (kind == 0 && index < c.species_names.size()) s = c.species_names[index];
        else if (kind == 1 && index < c.actions.size()) s = c.actions[index].name + ":" + c.actions[index].type;
        else if (kind == 2 && index < c.moves.size()) s = c.moves[index].name + ":" + c.moves[index].type;
        else if (kind == 3 && index < c.observables.size()) s = c.observables[index].name + ":" + c.observables[index].type;
        else throw pimc::PimcError(PIMC_ERR_ARG, "name index out of range");
        std::strncpy(buf, s.c_str(), cap - 1);
        buf[cap - 1] = '\0';
    });
}

int pimc_species_info(pimc_ctx* ctx, uint32_t s, uint32_t* n_part, uint32_t* offset, double* lambda) {
    return Guard(ctx, [&](pimc::Context& c) {
        if (s >= c.sys.S) throw pimc::PimcError(PIMC_ERR_ARG, "species index out of range");
        if (n_part) *n_part = c.sys.sp_n[s];
        if (offset) *offset = c.sys.sp_off[s];
        if (lambda) *lambda = c.sys.sp_lambda[s];
    });
}

int pimc_set_path(pimc_ctx* ctx, int which, const double* pos) {
    if (!pos || which < 0 || which > 2) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.SetPath(which, pos); });
}

int pimc_get_path(pimc_ctx* ctx, int which, double* pos) {
    if (!pos || which < 0 || which > 1) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.GetPath(which, pos); });
}

int pimc_get_rho_k(pimc_ctx* ctx, uint32_t species, double* out) {
    if (!out) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.GetRhoK(species, out); });
}

int pimc_get_kvecs(pimc_ctx* ctx, double* out) {
    if (!out) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.GetKVecs(out); });
}

int pimc_get_action(pimc_ctx* ctx, uint32_t action, uint32_t b0, uint32_t b1, const uint32_t* species, const uint32_t* particles,
                    uint32_t n_particles, uint32_t level, int mode, double* out) {
    if (!out || (n_particles && (!species || !particles))) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { *out = c.GetAction(action, b0, b1, species, particles, n_particles, level, mode); });
}

int pimc_get_action_gradient(pimc_ctx* ctx, uint32_t action, uint32_t b0, uint32_t b1, const uint32_t* species,
                             const uint32_t* particles, uint32_t n_particles, uint32_t level, int mode, double* out) {
    if (!out || (n_particles && (!species || !particles))) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        double g[3];
        c.GetActionGradient(action, b0, b1, species, particles, n_particles, level, mode, g);
        for (uint32_t d = 0; d < c.sys.n_d; ++d) out[d] = g[d];
    });
}

int pimc_get_action_gradient_exact(pimc_ctx* ctx, uint32_t action, uint32_t b0, uint32_t b1, const uint32_t* species,
                                   const uint32_t* particles, uint32_t n_particles, uint32_t level, int mode, double* out) {
    if (!out || (n_particles && (!species || !particles))) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        double g[3];
        c.ActionGradientAdjoint(action, b0, b1, species, particles, n_particles, level, mode, g);
        for (uint32_t d = 0; d < c.sys.n_d; ++d) out[d] = g[d];
    });
}

int pimc_set_precision(pimc_ctx* ctx, int bits) {
    return Guard(ctx, [&](pimc::Context& c) { c.SetPrecision(bits); });
}

int pimc_total_action(pimc_ctx* ctx, int action, int mode, double* out) {
    if (!out) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { *out = c.TotalAction(action, mode); });
}

int pimc_action_gradient_path(pimc_ctx* ctx, int action, int mode, double* grad) {
    if (!grad) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.ActionGradientPath(action, mode, grad); });
}

int pimc_dactiondbeta(pimc_ctx* ctx, uint32_t action, double* out) {
    if (!out) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { *out = c.DActionDBeta(action); });
}

int pimc_potential(pimc_ctx* ctx, uint32_t action, double* out) {
    if (!out) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { *out = c.Potential(action); });
}

int pimc_virial_energy(pimc_ctx* ctx, uint32_t action, double window, double* out) {
    if (!out || !(window >= 1.)) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { *out = c.VirialEnergy(action, window); });
}

int pimc_move_attempts(pimc_ctx* ctx, uint32_t move, uint64_t n) {
    return Guard(ctx, [&](pimc::Context& c) { c.MoveAttempts(move, n); });
}

int pimc_sweep(pimc_ctx* ctx, const uint32_t* moves, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep) {
    if (n_entries && (!moves || !counts)) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.Sweep(moves, counts, n_entries, n_rep); });
}

int pimc_sweep_chains(pimc_ctx** ctxs, uint32_t n_ctx, const uint32_t* moves, const uint64_t* counts, uint32_t n_entries, uint64_t n_rep) {
    if (!ctxs || n_ctx == 0 || (n_entries && (!moves || !counts))) return PIMC_ERR_ARG;
    for (uint32_t i = 0; i < n_ctx; ++i)
        if (!ctxs[i] || !ctxs[i]->c) return PIMC_ERR_ARG;
    return Guard(ctxs[0], [&](pimc::Context&) {
        std::vector<pimc::Context*> cs(n_ctx);
        for (uint32_t i = 0; i < n_ctx; ++i) cs[i] = ctxs[i]->c.get();
        pimc::SweepChains(cs, moves, counts, n_entries, n_rep);
    });
}

int pimc_move_stats(pimc_ctx* ctx, uint32_t move, uint64_t* out) {
    if (!out) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        if (move >= c.moves.size()) throw pimc::PimcError(PIMC_ERR_ARG, "move index out of range");
        out[0] = c.moves[move].attempts;
        out[1] = c.moves[move].block_attempt;
        out[2] = c.moves[move].block_accept;
        out[3] = c.moves[move].total_accept;
        out[4] = c.moves[move].total_level0;
    });
}

int pimc_get_perm(pimc_ctx* ctx, uint32_t species, uint32_t* perm) {
    if (!perm) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.GetPerm(species, perm); });
}

int pimc_set_perm(pimc_ctx* ctx, uint32_t species, const uint32_t* perm) {
    if (!perm) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.SetPerm(species, perm); });
}

int pimc_perm_stats(pimc_ctx* ctx, uint32_t move, uint64_t* out, size_t cap) {
    if (!out) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        if (move >= c.moves.size()) throw pimc::PimcError(PIMC_ERR_ARG, "move index out of range");
        const auto& mh = c.moves[move];
        if (mh.kind != 2 && mh.kind != 3) throw pimc::PimcError(PIMC_ERR_ARG, "not a permuting move");
        const size_t N = mh.perm_attempt.size();
        if (cap < 2 * N) throw pimc::PimcError(PIMC_ERR_ARG, "output shorter than twice the particle count");
        for (size_t i = 0; i < N; ++i) {
            out[i] = mh.perm_attempt[i];
            out[N + i] = mh.perm_accept[i];
        }
    });
}

int pimc_observable_accumulate(pimc_ctx* ctx, uint32_t observable) {
    return Guard(ctx, [&](pimc::Context& c) { c.ObservableAccumulate(observable); });
}

int pimc_observable_block(pimc_ctx* ctx, uint32_t observable, double* out, size_t cap, size_t* n) {
    if (!n || (cap && !out)) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        auto v = c.ObservableBlock(observable);
        *n = v.size();
        for (size_t i = 0; i < v.size() && i < cap; ++i) out[i] = v[i];
    });
}

int pimc_run(pimc_ctx* ctx) {
    return Guard(ctx, [&](pimc::Context& c) { c.Run(); });
}

int pimc_write_output(pimc_ctx* ctx, const char* path) {
    if (!path) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.WriteOutput(path); });
}

int pimc_n_blocks(pimc_ctx* ctx, uint32_t observable, size_t* n) {
    if (!n) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        if (observable >= c.blocks.size()) throw pimc::PimcError(PIMC_ERR_ARG, "observable index out of range");
        *n = c.blocks[observable].size();
    });
}

int pimc_get_block(pimc_ctx* ctx, uint32_t observable, size_t block, double* out, size_t cap, size_t* n) {
    if (!n || (cap && !out)) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) {
        if (observable >= c.blocks.size() || block >= c.blocks[observable].size())
            throw pimc::PimcError(PIMC_ERR_ARG, "block index out of range");
        const auto& v = c.blocks[observable][block];
        *n = v.size();
        for (size_t i = 0; i < v.size() && i < cap; ++i) out[i] = v[i];
    });
}

int pimc_synchronize(pimc_ctx* ctx) {
    return Guard(ctx, [&](pimc::Context& c) {
        c.Sync();
        c.CheckDeviceError();
    });
}

int pimc_set_sweep_grid(pimc_ctx* ctx, int grid) {
    return Guard(ctx, [&](pimc::Context& c) { c.sweep_grid = grid < 0 ? 0 : grid; });
}

int pimc_set_sweep_wave(pimc_ctx* ctx, int wave) {
    if (wave < 0 || wave > 8) return PIMC_ERR_ARG;
    return Guard(ctx, [&](pimc::Context& c) { c.sweep_wave = wave; });
}

int pimc_set_timeout_ns(pimc_ctx* ctx, uint64_t ns) {
    return Guard(ctx, [&](pimc::Context& c) { c.timeout_ns = ns; });
}

int pimc_check_wait_limit(pimc_ctx* ctx, uint64_t timeout_ns, uint64_t* waited_ns) {
    return Guard(ctx, [&](pimc::Context& c) { c.CheckWaitLimit(timeout_ns, waited_ns); });
}

void* pimc_stream(pimc_ctx* ctx) { return ctx && ctx->c ? (void*)ctx->c->stream : nullptr; }

int pimc_sweep_timing(pimc_ctx* ctx, int enable, uint64_t* cycles) {
    return Guard(ctx, [&](pimc::Context& c) {
        if (cycles) {
            for (int i = 0; i < pimc::kSweepTimingSlots; ++i) cycles[i] = 0;
            if (c.phase_buf) {
                pimc::CudaCheck(cudaMemcpy(cycles, c.phase_buf->ptr, pimc::kSweepTimingSlots * sizeof(uint64_t), cudaMemcpyDeviceToHost),
                                "read phase timing");
            }
        }
        if (enable >= 0) {
            c.phase_timing = enable != 0;
            if (c.phase_buf) pimc::CudaCheck(cudaMemset(c.phase_buf->ptr, 0, pimc::kSweepTimingSlots * sizeof(uint64_t)), "reset phase timing");
        }
    });
}

}  // extern "C"
