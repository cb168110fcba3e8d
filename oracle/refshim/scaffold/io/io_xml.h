// Reference build shim (test infrastructure): the XML `Input` class simpimc's headers read their
// configuration through (scaffold submodule, absent from the checkout). It wraps this repository's
// XML reader (simpimc_gb300/src/framework/input.h) behind the names the reference calls: Load,
// GetAttribute<T>(name[, default]), GetChild, GetChildList([name]), GetName, GetString and the
// `node.name` member that reads "null" for a missing child (framework_class.h:86).
#pragma once

#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../../../simpimc_gb300/src/framework/input.h"

namespace scaffold {
namespace io {

class Input {
   public:
    struct Node {
        std::string name = "null";
    } node;

    Input() = default;
    explicit Input(const pimc::Input& in) : in_(in) { node.name = in.GetName(); }

    void Load(const std::string& file) {
        std::ifstream f(file);
        std::stringstream ss;
        ss << f.rdbuf();
        text_ = ss.str();
        *this = FromText(text_);
    }
    static Input FromText(const std::string& text) {
        Input r(pimc::Input::FromString(text));
        r.text_ = text;
        return r;
    }
    template <class T>
    T GetAttribute(const std::string& key) const { return in_.GetAttribute<T>(key); }
    template <class T>
    T GetAttribute(const std::string& key, const T& dflt) const { return in_.GetAttribute<T>(key, dflt); }
    Input GetChild(const std::string& name) const { return Input(in_.GetChild(name)); }
    std::vector<Input> GetChildList(const std::string& name) const {
        std::vector<Input> out;
        for (auto& c : in_.GetChildList(name)) out.emplace_back(c);
        return out;
    }
    std::vector<Input> GetChildList() const {
        std::vector<Input> out;
        for (auto& c : in_.GetChildList()) out.emplace_back(c);
        return out;
    }
    std::string GetName() const { return in_.GetName(); }
    std::string GetString() const { return text_; }

   private:
    pimc::Input in_;
    std::string text_;
};

}  // namespace io
}  // namespace scaffold
