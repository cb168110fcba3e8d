// Run output and restart.
//
// The reference writes its output through IO (HDF5) under fixed dataset paths: Moves/<name>/*
// (move_class.h:49-53, 80-94; bisect_class.h:193-213) and Observables/<name>/* (observable_class.h:
// 79-88; energy_class.h:232-272; pair_correlation_class.h:76-120; structure_factor_class.h:56-82;
// path_dump_class.h:28-66), one value appended per Write event to its extendable datasets. HDF5 is
// not part of this build: the same paths are written to the table container of table_io.h, a
// dataset appended per Write stored as the flat concatenation of its appended values. A species
// with init_type="Restart" reads the last path dump back (species_class.h:336-377).
#include <cstdio>
#include <fstream>
#include <sstream>

#include "context.h"
#include "table_io.h"

namespace pimc {

namespace {

class Writer {
   public:
    explicit Writer(const std::string& path) : f_(path) {
        if (!f_) throw PimcError(kErrInput, "cannot open output file '" + path + "'");
        f_ << "# simpimc run output: '<dataset> <count>' then the values, or '<dataset> str' then a line\n";
    }
    void Str(const std::string& key, const std::string& v) {
        if (v.find('\n') != std::string::npos) throw PimcError(kErrArg, "string dataset spans lines");
        f_ << key << " str\n" << v << "\n";
    }
    void Num(const std::string& key, double v) { Vec(key, std::vector<double>{v}); }
    void Vec(const std::string& key, const std::vector<double>& v) {
        f_ << key << " " << v.size() << "\n";
        char buf[32];
        for (size_t i = 0; i < v.size(); ++i) {
            std::snprintf(buf, sizeof(buf), "%.17g", v[i]);
            f_ << buf << ((i % 4 == 3 || i + 1 == v.size()) ? "\n" : " ");
        }
    }
    void Close() {
        f_.close();
        if (!f_) throw PimcError(kErrInput, "writing the output file failed");
    }

   private:
    std::ofstream f_;
};

}  // namespace

void Context::WriteOutput(const std::string& path) {
    Writer w(path);
    for (const auto& mh : moves) {
        const std::string pre = "Moves/" + mh.name + "/";
        w.Str(pre + "type", mh.type);
        w.Str(pre + "data_type", "scalar");
        w.Vec(pre + "n_attempt", mh.out_attempt);
        w.Vec(pre + "n_accept", mh.out_accept);
        w.Vec(pre + "x", mh.out_ratio);
        if (mh.adaptive) w.Vec(pre + "n_level", mh.out_level);
        if (mh.kind == 2 || mh.kind == 3) {  // perm_bisect_class.h:119-132
            w.Num(pre + "n_perm_type", (double)mh.perm_n_type_out);
            std::vector<double> pa, pc;
            for (const auto& v : mh.out_perm_attempt) pa.insert(pa.end(), v.begin(), v.end());
            for (const auto& v : mh.out_perm_accept) pc.insert(pc.end(), v.begin(), v.end());
            w.Vec(pre + "perm_attempt", pa);
            w.Vec(pre + "perm_accept", pc);
        }
    }
    for (size_t oi = 0; oi < observables.size(); ++oi) {
        const ObservableHost& o = observables[oi];
        const std::string pre = "Observables/" + o.name + "/";
        w.Str(pre + "type", o.type);
        w.Str(pre + "data_type", (o.kind == 1 || o.kind == 2) ? "histogram" : (o.kind == 5 ? "scalar" : "none"));
        const auto& bl = blocks[oi];
        if (o.kind == 0) {
            // block layout: E, the per-action energies, then (with measure_potential) V and the potentials
            const size_t na = actions.size();
            auto column = [&](size_t c) {
                std::vector<double> v;
                for (const auto& b : bl) v.push_back(c < b.size() ? b[c] : 0.);
                return v;
            };
            w.Vec(pre + "total/x", column(0));
            w.Str(pre + "total/data_type", "scalar");
            for (size_t i = 0; i < na; ++i) {
                w.Vec(pre + actions[i].name + "/x", column(1 + i));
                w.Str(pre + actions[i].name + "/data_type", "scalar");
            }
            if (o.measure_potential) {
                w.Vec(pre + "v_total/x", column(1 + na));
                w.Str(pre + "v_total/data_type", "scalar");
                for (size_t i = 0; i < na; ++i) {
                    w.Vec(pre + "v_" + actions[i].name + "/x", column(2 + na + i));
                    w.Str(pre + "v_" + actions[i].name + "/data_type", "scalar");
                }
            }
        } else if (o.kind == 1) {
            w.Str(pre + "species_a", species_names[o.sa]);
            w.Str(pre + "species_b", species_names[o.sb]);
            w.Num(pre + "r_min", o.r_min);
            w.Num(pre + "r_max", o.r_max);
            w.Num(pre + "n_r", (double)o.n_r);
            std::vector<double> rs(o.n_r - 1);  // pair_correlation_class.h:64-74
            for (uint32_t i = 0; i + 1 < o.n_r; ++i) {
                const double r1 = o.r_min + i * o.dr, r2 = o.r_min + (i + 1) * o.dr;
                if (sys.n_d == 3) rs[i] = 0.75 * (r2 * r2 * r2 * r2 - r1 * r1 * r1 * r1) / (r2 * r2 * r2 - r1 * r1 * r1);
                else if (sys.n_d == 2) rs[i] = (r2 * r2 * r2 - r1 * r1 * r1) / (r2 * r2 - r1 * r1);
                else rs[i] = 0.5 * (r2 - r1);
            }
            w.Vec(pre + "x", rs);
            std::vector<double> y;
            for (const auto& b : bl) y.insert(y.end(), b.begin(), b.end());
            w.Vec(pre + "y", y);
        } else if (o.kind == 2) {
            w.Str(pre + "species_a", species_names[o.sa]);
            w.Str(pre + "species_b", species_names[o.sb]);
            w.Num(pre + "k_cut", o.k_cut);
            std::vector<double> kv((size_t)sys.K * sys.n_d), x(sys.K);
            if (sys.K) GetKVecs(kv.data());
            for (uint32_t k = 0; k < sys.K; ++k) {
                double s = 0.;
                for (uint32_t d = 0; d < sys.n_d; ++d) s += kv[(size_t)k * sys.n_d + d] * kv[(size_t)k * sys.n_d + d];
                x[k] = std::sqrt(s);
            }
            w.Vec(pre + "x", x);
            std::vector<double> y;
            for (const auto& b : bl) y.insert(y.end(), b.begin(), b.end());
            w.Vec(pre + "y", y);
        } else if (o.kind == 5) {
            std::vector<double> x;
            for (const auto& b : bl) x.push_back(b.empty() ? 0. : b[0]);
            w.Vec(pre + "x", x);
        } else if (o.kind == 6) {
            // permutation_class.h:36-73, 89-111
            const uint32_t n = sys.sp_n[o.species];
            w.Str(pre + "species", species_names[o.species]);
            w.Num(pre + "sector_max", (double)o.sector_max);
            w.Str(pre + "sectors/data_type", "pairs");
            std::vector<double> xs(o.partitions.size()), poss((size_t)n * o.partitions.size(), 0.);
            for (size_t i = 0; i < o.partitions.size(); ++i) {
                xs[i] = (double)i;
                for (uint32_t len : o.partitions[i]) poss[(size_t)(len - 1) * o.partitions.size() + i] += 1.;  // (n, n_perm) row-major
            }
            w.Vec(pre + "sectors/x", xs);
            w.Vec(pre + "sectors/possPerms", poss);
            w.Str(pre + "cycles/data_type", "histogram");
            std::vector<double> cx(n), cy, sy;
            for (uint32_t i = 0; i < n; ++i) cx[i] = i + 1.;
            for (const auto& b : bl) {
                cy.insert(cy.end(), b.begin(), b.begin() + std::min<size_t>(n, b.size()));
                if (b.size() > n) sy.insert(sy.end(), b.begin() + n, b.end());
            }
            w.Vec(pre + "cycles/x", cx);
            w.Vec(pre + "cycles/y", cy);
            w.Vec(pre + "sectors/y", sy);
        } else if (o.kind == 4) {
            for (uint32_t sp = 0; sp < sys.S; ++sp) {
                const std::string spre = pre + species_names[sp] + "/";
                const auto& dumps = o.dumps[sp];
                w.Num(spre + "n_dump", (double)dumps.size());
                std::vector<double> pos, perm;
                for (const auto& d : dumps) pos.insert(pos.end(), d.begin(), d.end());
                for (const auto& d : o.dump_perms[sp]) perm.insert(perm.end(), d.begin(), d.end());
                w.Vec(spre + "positions", pos);
                w.Vec(spre + "permutation", perm);
            }
        }
    }
    w.Close();
}

void Context::ApplyRestarts() {
    if (restarts.empty()) return;
    std::vector<double> host((size_t)sys.n_total * sys.M * sys.n_d, 0.);
    GetPath(0, host.data());  // species not restarted keep their positions
    std::vector<std::pair<uint32_t, std::vector<uint32_t>>> new_perms;
    for (const auto& r : restarts) {
        TableFile t = TableFile::Load(r.file);
        const std::string pre = "Observables/" + r.dump_name + "/" + species_names[r.species] + "/";
        const uint32_t n_dump = (uint32_t)t.Scalar(pre + "n_dump");
        const auto& pos = t.Vec(pre + "positions");
        const size_t per = (size_t)sys.sp_n[r.species] * sys.M * sys.n_d;
        if (n_dump == 0 || pos.size() < per * n_dump)
            throw PimcError(kErrInput, "restart file '" + r.file + "': no complete path dump for species " + species_names[r.species]);
        // the last dump's permutation (species_class.h:366-376): next particle at the closure,
        // checked against the recorded previous particles
        const auto& perm = t.Vec(pre + "permutation");
        const uint32_t N = sys.sp_n[r.species];
        std::vector<uint32_t> next(N);
        for (uint32_t p = 0; p < N; ++p) {
            const size_t at = ((size_t)(n_dump - 1) * N + p) * 2;
            if (at + 1 >= perm.size() || !(perm[at + 1] >= 0.) || perm[at + 1] >= N)
                throw PimcError(kErrInput, "restart file '" + r.file + "': incomplete permutation");
            next[p] = (uint32_t)perm[at + 1];
        }
        for (uint32_t p = 0; p < N; ++p)
            if (perm[((size_t)(n_dump - 1) * N + next[p]) * 2] != p)
                throw PimcError(kErrInput, "restart file '" + r.file + "': permutation columns disagree");
        new_perms.push_back({r.species, next});
        // positions(d, p n_bead + b, n_dump - 1) of the reference's cube read (species_class.h:354-364)
        std::copy(pos.begin() + per * (n_dump - 1), pos.begin() + per * n_dump, host.begin() + (size_t)sys.sp_off[r.species] * sys.M * sys.n_d);
    }
    SetPath(2, host.data());
    for (const auto& np : new_perms) SetPerm(np.first, np.second.data());
}

}  // namespace pimc
