// Reference harness (test infrastructure): simpimc's own action, move and observable classes,
// compiled from the reference checkout's unmodified headers against the shim in oracle/refshim/
// (which stands in for the absent scaffold, Armadillo, HDF5 and einspline). It exposes the same
// C surface as the oracle (oracle/oracle.cc) so tests can check the oracle, and through fixtures
// the GPU library, against the reference code itself. Built by oracle/build_ref.sh into
// oracle/_ref/; never part of the product.
//
// Set-up follows Simulation's constructor (framework/simulation_class.h:16-39) with the factories
// of actions.h, moves.h and observables.h restricted to the hot path's classes: Kinetic,
// HarmonicTrap, BarePairAction, IlkkaPairAction, DavidPairAction; Bisect, PermBisectIterative,
// PermBisectTable; Energy, PairCorrelation, StructureFactor, Sign, PathDump. Species start as init_type "Line" (species_class.h:311-321) and take their
// positions from refsim_set_path. Move draws are scripted (refshim/scaffold/rng/rng.h).
#include <sys/time.h>

#include <algorithm>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include <scaffold/algorithm/algorithm.h>
#include <scaffold/io/io_hdf5.h>
#include <scaffold/io/io_xml.h>
#include <scaffold/matrix/matrix.h>
#include <scaffold/rng/rng.h>

using namespace scaffold::matrix;
using namespace scaffold::algorithm;
using namespace scaffold::io;
using namespace scaffold::rand;

#include "actions/pair_action/bare_pair_action_class.h"
#include "actions/pair_action/david_pair_action_class.h"
#include "actions/pair_action/ilkka_pair_action_class.h"
#include "actions/single_action/kinetic_class.h"
#include "actions/single_action/trap_class.h"
#include "data_structures/path_class.h"
#include "events/moves/single_species_move/bisect/bisect_class.h"
#include "events/moves/single_species_move/bisect/perm_bisect/perm_bisect_iterative_class.h"
#include "events/moves/single_species_move/bisect/perm_bisect/perm_bisect_table_class.h"
#include "events/observables/energy_class.h"
#include "events/observables/pair_correlation_class.h"
#include "events/observables/path_dump_class.h"
#include "events/observables/sign_class.h"
#include "events/observables/structure_factor_class.h"

namespace {

std::string g_err;

struct RefSim {
    Input in;
    IO out;
    RNG rng;
    std::unique_ptr<Path> path;
    std::vector<std::shared_ptr<Action>> actions;
    std::vector<std::shared_ptr<Move>> moves;
    std::vector<std::shared_ptr<Observable>> observables;
    std::vector<std::string> move_names, obs_names, obs_types;
};

std::string ReplaceAll(std::string s, const std::string& a, const std::string& b) {
    for (size_t i = s.find(a); i != std::string::npos; i = s.find(a, i + b.size())) s.replace(i, a.size(), b);
    return s;
}

std::shared_ptr<Action> MakeAction(Input& in, IO& out, Path& path) {
    std::string type = in.GetAttribute<std::string>("type");
    if (type == "Kinetic") return std::make_shared<Kinetic>(path, in, out);
    if (type == "HarmonicTrap") return std::make_shared<Trap>(path, in, out);
    if (type == "BarePairAction") return std::make_shared<BarePairAction>(path, in, out);
    if (type == "DavidPairAction") return std::make_shared<DavidPairAction>(path, in, out);
    if (type == "IlkkaPairAction") return std::make_shared<IlkkaPairAction>(path, in, out);
    throw std::runtime_error("reference harness: action type " + type + " not built");
}

std::vector<std::pair<std::shared_ptr<Species>, uint32_t>> Parts(RefSim& s, const uint32_t* sp, const uint32_t* p, uint32_t n) {
    std::vector<std::pair<std::shared_ptr<Species>, uint32_t>> out;
    auto& all = s.path->GetSpecies();
    for (uint32_t i = 0; i < n; ++i) out.emplace_back(all.at(sp[i]), p[i]);
    return out;
}

template <class F>
int Guard(F f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_err = e.what();
        return -1;
    }
}

RefSim* S(void* h) { return static_cast<RefSim*>(h); }

// Pointers to the protected counters of Move (move_class.h:11-12) and the level of Bisect
// (bisect_class.h:19), taken through derived classes so the harness can read them between Write
// events without changing the reference's classes.
struct MoveCounterAccess : Move {
    static uint32_t Move::*Attempts() { return &MoveCounterAccess::n_attempt; }
    static uint32_t Move::*Accepts() { return &MoveCounterAccess::n_accept; }
};
struct BisectLevelAccess : Bisect {
    static uint32_t Bisect::*Level() { return &BisectLevelAccess::n_level; }
};
// The per-cycle-length counters of PermBisect (perm_bisect_class.h:25-26).
struct PermCounterAccess : PermBisect {
    static vec<uint32_t> PermBisect::*Attempts() { return &PermCounterAccess::perm_attempt; }
    static vec<uint32_t> PermBisect::*Accepts() { return &PermCounterAccess::perm_accept; }
};

}  // namespace

extern "C" {

const char* refsim_last_error() { return g_err.c_str(); }

int refsim_create(const char* xml, const char* dir, void** out) {
    return Guard([&] {
        auto s = std::make_unique<RefSim>();
        scaffold::io::base_dir() = dir ? dir : "";
        std::string text = ReplaceAll(xml, "init_type=\"File\"", "init_type=\"Line\"");
        s->in = Input::FromText(text);
        s->rng = RNG(s->in.GetChild("RNG").GetAttribute<int>("seed", 0));
        s->path.reset(new Path(0, s->in, s->out, s->rng));
        for (auto& a : s->in.GetChild("Actions").GetChildList("Action")) s->actions.push_back(MakeAction(a, s->out, *s->path));
        for (auto& m : s->in.GetChild("Moves").GetChildList("Move")) {
            const std::string type = m.GetAttribute<std::string>("type");
            if (type == "Bisect") s->moves.push_back(std::make_shared<Bisect>(*s->path, s->rng, s->actions, m, s->out));
            else if (type == "PermBisectIterative") s->moves.push_back(std::make_shared<PermBisectIterative>(*s->path, s->rng, s->actions, m, s->out));
            else if (type == "PermBisectTable") s->moves.push_back(std::make_shared<PermBisectTable>(*s->path, s->rng, s->actions, m, s->out));
            else continue;
            s->move_names.push_back(m.GetAttribute<std::string>("name"));
        }
        for (auto& o : s->in.GetChild("Observables").GetChildList("Observable")) {
            std::string type = o.GetAttribute<std::string>("type");
            std::shared_ptr<Observable> ob;
            if (type == "Energy") ob = std::make_shared<Energy>(*s->path, s->actions, o, s->out);
            else if (type == "PairCorrelation") ob = std::make_shared<PairCorrelation>(*s->path, o, s->out);
            else if (type == "StructureFactor") ob = std::make_shared<StructureFactor>(*s->path, o, s->out);
            else if (type == "Sign") ob = std::make_shared<Sign>(*s->path, o, s->out);
            else if (type == "PathDump") ob = std::make_shared<PathDump>(*s->path, o, s->out);
            else continue;
            s->observables.push_back(ob);
            s->obs_names.push_back(o.GetAttribute<std::string>("name"));
            s->obs_types.push_back(type);
        }
        *out = s.release();
    });
}

void refsim_destroy(void* h) { delete S(h); }

/// counts[4] = {species, total particles, beads, stored k-vectors}
int refsim_info(void* h, uint32_t* out) {
    return Guard([&] {
        auto& sp = S(h)->path->GetSpecies();
        uint32_t n = 0;
        for (auto& s : sp) n += s->GetNPart();
        out[0] = (uint32_t)sp.size();
        out[1] = n;
        out[2] = S(h)->path->GetNBead();
        out[3] = (uint32_t)S(h)->path->ks.vecs.size();
    });
}

/// Positions from pos[g][b][d] (g over all species in order) into the stored copy (which = 0), the
/// working copy (1, Bead::SetR in NEW_MODE, bead_class.h:101) or both (2, then every species'
/// densities, Species::InitRhoK, species_class.h:380-403).
int refsim_set_path(void* h, int which, const double* pos) {
    return Guard([&] {
        Path& path = *S(h)->path;
        const uint32_t M = path.GetNBead(), nd = path.GetND();
        path.SetMode(which == 0 ? OLD_MODE : NEW_MODE);
        size_t g = 0;
        for (auto& s : path.GetSpecies()) {
            for (uint32_t p = 0; p < s->GetNPart(); ++p, ++g)
                for (uint32_t b = 0; b < M; ++b) {
                    vec<double> r(nd);
                    for (uint32_t d = 0; d < nd; ++d) r(d) = pos[(g * M + b) * nd + d];
                    s->GetBead(p, b)->SetR(r);
                    if (which == 2) s->GetBead(p, b)->StoreR();
                }
            if (which == 2) s->InitRhoK();
            s->SetNeedUpdateRhoK(true);
        }
        path.SetMode(NEW_MODE);
    });
}

int refsim_get_path(void* h, int which, double* pos) {
    return Guard([&] {
        Path& path = *S(h)->path;
        const uint32_t M = path.GetNBead(), nd = path.GetND();
        const ModeType keep = path.GetMode();
        path.SetMode(which ? NEW_MODE : OLD_MODE);
        size_t g = 0;
        for (auto& s : path.GetSpecies())
            for (uint32_t p = 0; p < s->GetNPart(); ++p, ++g)
                for (uint32_t b = 0; b < M; ++b) {
                    const vec<double>& r = s->GetBead(p, b)->GetR();
                    for (uint32_t d = 0; d < nd; ++d) pos[(g * M + b) * nd + d] = r(d);
                }
        path.SetMode(keep);
    });
}

/// Per-slice densities of one species, [M][K][re, im], of the chosen copy.
int refsim_get_rho_k(void* h, uint32_t species, int which, double* out) {
    return Guard([&] {
        Path& path = *S(h)->path;
        auto& s = path.GetSpecies().at(species);
        const ModeType keep = path.GetMode();
        path.SetMode(which ? NEW_MODE : OLD_MODE);
        auto& rho = s->GetRhoK();
        const size_t K = path.ks.vecs.size();
        for (uint32_t b = 0; b < path.GetNBead(); ++b)
            for (size_t k = 0; k < K; ++k) {
                out[(b * K + k) * 2] = rho(b)(k).real();
                out[(b * K + k) * 2 + 1] = rho(b)(k).imag();
            }
        path.SetMode(keep);
    });
}

int refsim_kvecs(void* h, double* out) {
    return Guard([&] {
        Path& path = *S(h)->path;
        for (size_t k = 0; k < path.ks.vecs.size(); ++k)
            for (uint32_t d = 0; d < path.GetND(); ++d) out[k * path.GetND() + d] = path.ks.vecs[k](d);
    });
}

/// The NEW-mode density latch of every species set again (species_class.h:25, 424).
int refsim_reset_rho_k_latch(void* h) {
    return Guard([&] {
        for (auto& s : S(h)->path->GetSpecies()) s->SetNeedUpdateRhoK(true);
    });
}

int refsim_get_action(void* h, uint32_t a, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n, uint32_t level,
                      int mode, double* out) {
    return Guard([&] {
        RefSim& s = *S(h);
        auto parts = Parts(s, sp, p, n);
        s.path->SetMode(mode ? NEW_MODE : OLD_MODE);
        *out = s.actions.at(a)->GetAction(b0, b1, parts, level);
        s.path->SetMode(NEW_MODE);
    });
}

int refsim_get_action_gradient(void* h, uint32_t a, uint32_t b0, uint32_t b1, const uint32_t* sp, const uint32_t* p, uint32_t n,
                               uint32_t level, int mode, double* out) {
    return Guard([&] {
        RefSim& s = *S(h);
        auto parts = Parts(s, sp, p, n);
        s.path->SetMode(mode ? NEW_MODE : OLD_MODE);
        vec<double> g = s.actions.at(a)->GetActionGradient(b0, b1, parts, level);
        s.path->SetMode(NEW_MODE);
        for (uint32_t d = 0; d < s.path->GetND(); ++d) out[d] = g(d);
    });
}

int refsim_dactiondbeta(void* h, uint32_t a, double* out) {
    return Guard([&] { *out = S(h)->actions.at(a)->DActionDBeta(); });
}

int refsim_potential(void* h, uint32_t a, double* out) {
    return Guard([&] { *out = S(h)->actions.at(a)->Potential(); });
}

int refsim_virial_energy(void* h, uint32_t a, double window, double* out) {
    return Guard([&] { *out = S(h)->actions.at(a)->VirialEnergy(window); });
}

/// One Move::DoEvent of move m (move_class.h:61-77) with its draws: the particle and first bead
/// (0-based), `n_z` normal triples in sampling order and `n_u` level uniforms (top level first).
int refsim_move_attempt(void* h, uint32_t m, uint32_t particle, uint32_t bead0, const double* z, uint32_t n_z, const double* u,
                        uint32_t n_u) {
    return Guard([&] {
        RefSim& s = *S(h);
        s.rng.Clear();
        s.rng.QueueIndex(particle + 1);
        s.rng.QueueIndex(bead0 + 1);
        for (uint32_t i = 0; i < n_z; ++i) s.rng.QueueNormal({z[3 * i], z[3 * i + 1], z[3 * i + 2]});
        for (uint32_t i = 0; i < n_u; ++i) s.rng.QueueUniform(u[i]);
        s.moves.at(m)->DoEvent();
        s.rng.Clear();
    });
}

/// One Move::DoEvent of permuting move m (PermBisectIterative or PermBisectTable) with its draws:
/// the first bead (0-based), the cycle's first particle (iterative only; ignored otherwise),
/// `n_z` normal triples in sampling order (level, cycle particle, position along the path), the
/// `n_sel` uniforms of the cycle selection (iterative: continuation and choice of each step in
/// turn; table: the selection uniform) and the `n_u` uniforms drawn after sampling starts (level
/// tests, top level first, then the table's final test).
int refsim_perm_attempt(void* h, uint32_t m, uint32_t bead0, uint32_t particle, const double* z, uint32_t n_z, const double* sel,
                        uint32_t n_sel, const double* u, uint32_t n_u) {
    return Guard([&] {
        RefSim& s = *S(h);
        Move* mv = s.moves.at(m).get();
        const bool iterative = dynamic_cast<PermBisectIterative*>(mv) != nullptr;
        if (!iterative && !dynamic_cast<PermBisectTable*>(mv)) throw std::invalid_argument("not a permuting move");
        s.rng.Clear();
        s.rng.QueueIndex(bead0 + 1);
        if (iterative) s.rng.QueueIndex(particle + 1);
        for (uint32_t i = 0; i < n_z; ++i) s.rng.QueueNormal({z[3 * i], z[3 * i + 1], z[3 * i + 2]});
        for (uint32_t i = 0; i < n_sel; ++i) s.rng.QueueSelectionUniform(sel[i]);
        for (uint32_t i = 0; i < n_u; ++i) s.rng.QueueUniform(u[i]);
        mv->DoEvent();
        s.rng.Clear();
    });
}

/// out[2 N] = the permuting move's attempts, then accepts, per cycle length in its current block.
int refsim_perm_counters(void* h, uint32_t m, uint64_t* out) {
    return Guard([&] {
        auto* mv = dynamic_cast<PermBisect*>(S(h)->moves.at(m).get());
        if (!mv) throw std::invalid_argument("not a permuting move");
        const vec<uint32_t>& att = mv->*PermCounterAccess::Attempts();
        const vec<uint32_t>& acc = mv->*PermCounterAccess::Accepts();
        for (size_t i = 0; i < att.size(); ++i) {
            out[i] = att(i);
            out[att.size() + i] = acc(i);
        }
    });
}

/// out[p] = the particle whose slice-0 bead follows particle p's last bead (the committed links,
/// bead_class.h:107): the path permutation at the ring closure.
int refsim_get_perm(void* h, uint32_t species, uint32_t* out) {
    return Guard([&] {
        Path& path = *S(h)->path;
        auto& s = path.GetSpecies().at(species);
        const ModeType keep = path.GetMode();
        path.SetMode(OLD_MODE);
        for (uint32_t p = 0; p < s->GetNPart(); ++p) out[p] = s->GetBead(p, path.GetNBead() - 1)->GetNextBead(1)->GetP();
        path.SetMode(keep);
    });
}

/// out[3] = {attempts, accepts} of the move's current block and its bisection level.
int refsim_move_counters(void* h, uint32_t m, uint64_t* out) {
    return Guard([&] {
        Move& mv = *S(h)->moves.at(m);
        out[0] = mv.*MoveCounterAccess::Attempts();
        out[1] = mv.*MoveCounterAccess::Accepts();
        out[2] = static_cast<Bisect&>(mv).*BisectLevelAccess::Level();
    });
}

/// Move::Write (move_class.h:80-94, bisect_class.h:193-213): appends the block's counters to the
/// output, adapts the bisection level when the move is adaptive (bisect_class.h:142-155) and resets
/// the counters. out[3] = the appended {n_attempt, n_accept} and the level written with them (the
/// level in force before the adaptation; -1 when the move is not adaptive).
int refsim_move_write(void* h, uint32_t m, int64_t* out) {
    return Guard([&] {
        RefSim& s = *S(h);
        s.moves.at(m)->Write();
        const std::string pre = "Moves/" + s.move_names.at(m) + "/";
        out[0] = (int64_t)s.out.Appended(pre + "n_attempt")->back()[0];
        out[1] = (int64_t)s.out.Appended(pre + "n_accept")->back()[0];
        auto* lv = s.out.Appended(pre + "n_level");
        out[2] = lv ? (int64_t)lv->back()[0] : -1;
    });
}

int refsim_obs_accumulate(void* h, uint32_t o) {
    return Guard([&] { S(h)->observables.at(o)->DoEvent(); });
}

/// Observable::Write (observable_class.h:104), then the values it appended: Energy's total and
/// per-action energies in action order (energy_class.h:232-253); the y histogram of
/// PairCorrelation and StructureFactor. *n = 0 when the Write appended nothing (no measurement
/// since the last one).
int refsim_obs_write(void* h, uint32_t o, double* out, uint64_t cap, uint64_t* n) {
    return Guard([&] {
        RefSim& s = *S(h);
        const std::string pre = "Observables/" + s.obs_names.at(o) + "/";
        const std::string& type = s.obs_types[o];
        if (type == "PathDump") {  // per species: the dump's positions (d fastest, then bead, then particle), then (prev, next) per particle
            auto& species = s.path->GetSpecies();
            auto rows = [&]() -> size_t {
                auto* r = s.out.Appended(pre + species.at(0)->GetName() + "/positions");
                return r ? r->size() : 0;
            };
            const size_t before = rows();
            s.observables.at(o)->Write();
            *n = 0;
            if (rows() == before) return;
            std::vector<double> vals;
            for (auto& sp : species)
                for (const char* what : {"/positions", "/permutation"}) {
                    const auto& row = s.out.Appended(pre + sp->GetName() + what)->back();
                    vals.insert(vals.end(), row.begin(), row.end());
                }
            *n = vals.size();
            for (size_t i = 0; i < vals.size() && i < cap; ++i) out[i] = vals[i];
            return;
        }
        const std::string key = type == "Energy" ? pre + "total/x" : type == "Sign" ? pre + "x" : pre + "y";
        auto rows = [&]() -> size_t {
            auto* r = s.out.Appended(key);
            return r ? r->size() : 0;
        };
        const size_t before = rows();
        s.observables.at(o)->Write();
        *n = 0;
        if (rows() == before) return;
        std::vector<double> vals;
        if (s.obs_types[o] == "Energy") {
            vals.push_back(s.out.Appended(pre + "total/x")->back()[0]);
            for (auto& a : s.actions) {
                auto* r = s.out.Appended(pre + a->name + "/x");
                if (r) vals.push_back(r->back()[0]);
            }
        } else {
            vals = s.out.Appended(key)->back();
        }
        *n = vals.size();
        for (size_t i = 0; i < vals.size() && i < cap; ++i) out[i] = vals[i];
    });
}

}  // extern "C"
