// Reference build shim (test infrastructure): the `IO` class simpimc's headers write their output
// and read their pair-action tables through (scaffold submodule over HDF5, both absent here).
// - Reading: Load(file) opens a table written by this repository (the text container of
//   simpimc_gb300/src/framework/table_io.h, which keeps the reference's dataset paths); Read fills
//   scalars, strings, vec, mat and cube from a dataset in storage order. Relative file names resolve
//   against `base_dir()`, which the harness sets.
// - Writing: Write/CreateGroup keep nothing; CreateExtendableDataSet/AppendDataSet keep every
//   appended value per dataset path, so a harness can read the blocks an observable or move wrote.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "../../../../simpimc_gb300/src/framework/table_io.h"
#include "../matrix/matrix.h"

namespace scaffold {
namespace io {

inline std::string& base_dir() {
    static std::string d;
    return d;
}

inline std::string NormalisePath(const std::string& p) {
    std::string out;
    for (size_t i = 0; i < p.size(); ++i) {
        if (p[i] == '/' && (out.empty() || out.back() == '/')) continue;
        out.push_back(p[i]);
    }
    while (!out.empty() && out.back() == '/') out.pop_back();
    return out;
}

class IO {
   public:
    void Load(const std::string& file) {
        name_ = file;
        std::string path = file;
        if (!file.empty() && file[0] != '/' && !base_dir().empty()) path = base_dir() + "/" + file;
        std::ifstream probe(path);
        if (probe) table_ = std::make_shared<pimc::TableFile>(pimc::TableFile::Load(path));
    }
    void Create() {}
    void CreateGroup(const std::string&) {}
    template <class T>
    void Write(const std::string&, const T&) {}
    template <class T>
    void Rewrite(const std::string&, const T&) {}

    template <class T>
    void CreateExtendableDataSet(const std::string& prefix, const std::string& name, const T& v) {
        auto& rows = data_[NormalisePath(prefix + "/" + name)];
        rows.clear();
        rows.push_back(Flatten(v));
    }
    template <class T>
    void AppendDataSet(const std::string& prefix, const std::string& name, const T& v) {
        data_[NormalisePath(prefix + "/" + name)].push_back(Flatten(v));
    }
    /// Rows appended to an extendable dataset (harness access).
    const std::vector<std::vector<double>>* Appended(const std::string& path) const {
        auto it = data_.find(NormalisePath(path));
        return it == data_.end() ? nullptr : &it->second;
    }

    void Read(const std::string& p, std::string& v) { v = Table().String(NormalisePath(p)); }
    void Read(const std::string& p, double& v) { v = Table().Scalar(NormalisePath(p)); }
    void Read(const std::string& p, uint32_t& v) { v = (uint32_t)Table().Scalar(NormalisePath(p)); }
    void Read(const std::string& p, int& v) { v = (int)Table().Scalar(NormalisePath(p)); }
    template <class A>
    void Read(const std::string& p, A& a) {
        const auto& src = Table().Vec(NormalisePath(p));
        if (src.size() != a.size())
            throw pimc::InputError("table '" + name_ + "': dataset '" + p + "' has " + std::to_string(src.size()) + " values, want " +
                                   std::to_string(a.size()));
        for (size_t i = 0; i < src.size(); ++i) a.memptr()[i] = src[i];
    }

   private:
    std::string name_;
    std::shared_ptr<pimc::TableFile> table_;
    std::map<std::string, std::vector<std::vector<double>>> data_;

    const pimc::TableFile& Table() const {
        if (!table_) throw pimc::InputError("cannot open table '" + name_ + "'");
        return *table_;
    }
    template <class T>
    static std::vector<double> Flatten(const T& v) {
        if constexpr (std::is_arithmetic<T>::value) {
            return {(double)v};
        } else {
            std::vector<double> out;
            for (size_t i = 0; i < v.size(); ++i) out.push_back((double)v.memptr()[i]);
            return out;
        }
    }
};

}  // namespace io
}  // namespace scaffold
