// Pair-action table files.
//
// The reference loads pair-action tables from HDF5 files through `IO::Read(dataset_path, value)`
// (src/actions/pair_action/bare_pair_action_class.h:29-76). HDF5 is not part of this build, so the
// same datasets are stored in a plain text container that keeps the reference's dataset paths:
//
//     # comment
//     v/diag/n_r 1
//     1000
//     v/diag/r 1000
//     1.0e-4 ...
//
// Each record is "<dataset path> <count>" followed by <count> whitespace-separated numbers.
// Scalars are records of count 1. Numbers are written with 17 significant digits so that a
// round trip through the file is exact in double precision. A string dataset (the reference's
// names and type tags) is "<dataset path> str" followed by one line holding the string.
#pragma once

#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "input.h"

namespace pimc {

class TableFile {
   public:
    TableFile() = default;

    static TableFile Load(const std::string& path) {
        std::ifstream f(path);
        if (!f) throw InputError("cannot open pair-action table '" + path + "'");
        TableFile t;
        t.path_ = path;
        std::string line;
        std::string key;
        size_t want = 0;
        std::vector<double> vals;
        auto flush = [&]() {
            if (!key.empty()) {
                if (vals.size() != want)
                    throw InputError("table '" + path + "': dataset '" + key + "' has " + std::to_string(vals.size()) +
                                     " values, header says " + std::to_string(want));
                t.data_[key] = vals;
            }
            key.clear();
            vals.clear();
            want = 0;
        };
        while (std::getline(f, line)) {
            size_t h = line.find('#');
            if (h != std::string::npos) line.resize(h);
            std::istringstream ls(line);
            std::string tok;
            {
                // "<path> str": the next line is the string value
                std::istringstream peek(line);
                std::string k, c, extra;
                if ((key.empty() || vals.size() >= want) && (peek >> k >> c) && c == "str" && !(peek >> extra)) {
                    flush();
                    std::string v;
                    if (!std::getline(f, v)) throw InputError("table '" + path + "': string dataset '" + k + "' lacks its line");
                    t.strings_[k] = v;
                    continue;
                }
            }
            while (ls >> tok) {
                if (!key.empty() && vals.size() < want) {
                    char* end = nullptr;
                    double x = std::strtod(tok.c_str(), &end);
                    if (end == tok.c_str() || *end != '\0')
                        throw InputError("table '" + path + "': bad number '" + tok + "' in dataset '" + key + "'");
                    vals.push_back(x);
                    continue;
                }
                flush();
                key = tok;
                std::string cnt;
                if (!(ls >> cnt)) throw InputError("table '" + path + "': dataset '" + key + "' lacks a count");
                char* end = nullptr;
                long c = std::strtol(cnt.c_str(), &end, 10);
                if (end == cnt.c_str() || c < 0) throw InputError("table '" + path + "': bad count for '" + key + "'");
                want = static_cast<size_t>(c);
            }
        }
        flush();
        return t;
    }

    bool Has(const std::string& key) const { return data_.count(key) != 0; }
    bool HasString(const std::string& key) const { return strings_.count(key) != 0; }
    const std::string& String(const std::string& key) const {
        auto it = strings_.find(key);
        if (it == strings_.end()) throw InputError("table '" + path_ + "' has no string dataset '" + key + "'");
        return it->second;
    }

    const std::vector<double>& Vec(const std::string& key) const {
        auto it = data_.find(key);
        if (it == data_.end()) throw InputError("table '" + path_ + "' has no dataset '" + key + "'");
        return it->second;
    }

    double Scalar(const std::string& key) const {
        const auto& v = Vec(key);
        if (v.size() != 1) throw InputError("table '" + path_ + "': dataset '" + key + "' is not a scalar");
        return v[0];
    }

   private:
    std::string path_;
    std::map<std::string, std::vector<double>> data_;
    std::map<std::string, std::string> strings_;
};

}  // namespace pimc
