// XML input tree with the accessor surface simpimc's code reads its configuration through.
//
// The reference reads every setting through a small `Input` API (GetAttribute<T>(name[, default]),
// GetChild, GetChildList, GetName); call sites e.g. src/data_structures/path_class.h:25-62,
// src/actions/action_class.h:23-34, src/framework/simulation_class.h:16-39. This is a fresh,
// self-contained implementation of that surface over a minimal XML subset: elements, attributes,
// comments, processing instructions. Element text content is ignored (simpimc inputs carry none).
//
// Semantics kept from the reference: attribute names are case-sensitive; a missing attribute
// without a default is an error; a missing child yields an empty node named "null" (the
// reference tests `rng_in.node.name == "null"`, src/framework/framework_class.h:86).
#pragma once

#include <cctype>
#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace pimc {

struct InputError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct XmlNode {
    std::string name = "null";
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<std::shared_ptr<XmlNode>> children;
};

namespace detail {

class XmlParser {
   public:
    explicit XmlParser(const std::string& s) : s_(s), i_(0) {}

    std::shared_ptr<XmlNode> ParseDocument() {
        SkipMisc();
        if (i_ >= s_.size() || s_[i_] != '<') Fail("expected root element");
        auto root = ParseElement();
        SkipMisc();
        if (i_ != s_.size()) Fail("trailing content after root element");
        return root;
    }

   private:
    const std::string& s_;
    size_t i_;

    [[noreturn]] void Fail(const std::string& what) {
        size_t line = 1;
        for (size_t j = 0; j < i_ && j < s_.size(); ++j)
            if (s_[j] == '\n') ++line;
        throw InputError("XML parse error at line " + std::to_string(line) + ": " + what);
    }

    void SkipWs() {
        while (i_ < s_.size() && (s_[i_] == ' ' || s_[i_] == '\t' || s_[i_] == '\n' || s_[i_] == '\r')) ++i_;
    }

    bool StartsWith(const char* p) const { return s_.compare(i_, std::char_traits<char>::length(p), p) == 0; }

    void SkipUntil(const char* end) {
        size_t j = s_.find(end, i_);
        if (j == std::string::npos) Fail(std::string("unterminated construct, missing ") + end);
        i_ = j + std::char_traits<char>::length(end);
    }

    // Whitespace, comments, <?...?> and <!...> declarations.
    void SkipMisc() {
        for (;;) {
            SkipWs();
            if (StartsWith("<!--")) SkipUntil("-->");
            else if (StartsWith("<?")) SkipUntil("?>");
            else if (StartsWith("<!")) SkipUntil(">");
            else return;
        }
    }

    static bool NameChar(char c) {
        return std::isalnum(static_cast<unsigned char>(c)) || c == '_' || c == '-' || c == '.' || c == ':';
    }

    std::string ParseName() {
        size_t j = i_;
        while (i_ < s_.size() && NameChar(s_[i_])) ++i_;
        if (j == i_) Fail("expected a name");
        return s_.substr(j, i_ - j);
    }

    static std::string Unescape(const std::string& v) {
        std::string out;
        out.reserve(v.size());
        for (size_t k = 0; k < v.size(); ++k) {
            if (v[k] != '&') { out += v[k]; continue; }
            size_t e = v.find(';', k);
            if (e == std::string::npos) { out += v[k]; continue; }
            std::string ent = v.substr(k + 1, e - k - 1);
            if (ent == "lt") out += '<';
            else if (ent == "gt") out += '>';
            else if (ent == "amp") out += '&';
            else if (ent == "quot") out += '"';
            else if (ent == "apos") out += '\'';
            else { out += v.substr(k, e - k + 1); }
            k = e;
        }
        return out;
    }

    std::shared_ptr<XmlNode> ParseElement() {
        ++i_;  // '<'
        auto node = std::make_shared<XmlNode>();
        node->name = ParseName();
        for (;;) {
            SkipWs();
            if (i_ >= s_.size()) Fail("unterminated start tag <" + node->name);
            if (StartsWith("/>")) { i_ += 2; return node; }
            if (s_[i_] == '>') { ++i_; break; }
            std::string key = ParseName();
            SkipWs();
            if (i_ >= s_.size() || s_[i_] != '=') Fail("expected '=' after attribute " + key);
            ++i_;
            SkipWs();
            if (i_ >= s_.size() || (s_[i_] != '"' && s_[i_] != '\'')) Fail("expected quoted value for " + key);
            char q = s_[i_++];
            size_t e = s_.find(q, i_);
            if (e == std::string::npos) Fail("unterminated attribute value for " + key);
            node->attrs.emplace_back(key, Unescape(s_.substr(i_, e - i_)));
            i_ = e + 1;
        }
        // Content: children, comments, ignored text, then the matching end tag.
        for (;;) {
            size_t j = s_.find('<', i_);
            if (j == std::string::npos) Fail("missing end tag </" + node->name + ">");
            i_ = j;
            if (StartsWith("<!--")) { SkipUntil("-->"); continue; }
            if (StartsWith("<?")) { SkipUntil("?>"); continue; }
            if (StartsWith("</")) {
                i_ += 2;
                std::string end = ParseName();
                if (end != node->name) Fail("end tag </" + end + "> does not match <" + node->name + ">");
                SkipWs();
                if (i_ >= s_.size() || s_[i_] != '>') Fail("malformed end tag");
                ++i_;
                return node;
            }
            node->children.push_back(ParseElement());
        }
    }
};

template <class T>
inline T ConvertAttr(const std::string& v, const std::string& name);

template <>
inline std::string ConvertAttr<std::string>(const std::string& v, const std::string&) { return v; }

template <>
inline double ConvertAttr<double>(const std::string& v, const std::string& name) {
    char* end = nullptr;
    double x = std::strtod(v.c_str(), &end);
    if (end == v.c_str()) throw InputError("attribute '" + name + "' is not a number: '" + v + "'");
    return x;
}

template <>
inline int ConvertAttr<int>(const std::string& v, const std::string& name) {
    char* end = nullptr;
    long x = std::strtol(v.c_str(), &end, 10);
    if (end == v.c_str()) throw InputError("attribute '" + name + "' is not an integer: '" + v + "'");
    return static_cast<int>(x);
}

template <>
inline uint32_t ConvertAttr<uint32_t>(const std::string& v, const std::string& name) {
    // The reference reads some counts through a double (pair_correlation_class.h:60); accept "100.0".
    char* end = nullptr;
    double x = std::strtod(v.c_str(), &end);
    if (end == v.c_str() || x < 0) throw InputError("attribute '" + name + "' is not a non-negative integer: '" + v + "'");
    return static_cast<uint32_t>(x);
}

template <>
inline bool ConvertAttr<bool>(const std::string& v, const std::string& name) {
    if (v == "1" || v == "true" || v == "True") return true;
    if (v == "0" || v == "false" || v == "False") return false;
    throw InputError("attribute '" + name + "' is not a boolean: '" + v + "'");
}

}  // namespace detail

/// A view of one XML element (cheap to copy; shares the parsed tree).
class Input {
   public:
    Input() : node_(std::make_shared<XmlNode>()) {}
    explicit Input(std::shared_ptr<XmlNode> n) : node_(std::move(n)) {}

    static Input FromString(const std::string& text) {
        detail::XmlParser p(text);
        return Input(p.ParseDocument());
    }

    static Input FromFile(const std::string& path) {
        std::ifstream f(path);
        if (!f) throw InputError("cannot open input file '" + path + "'");
        std::stringstream ss;
        ss << f.rdbuf();
        return FromString(ss.str());
    }

    const std::string& GetName() const { return node_->name; }
    bool IsNull() const { return node_->name == "null"; }

    bool HasAttribute(const std::string& key) const {
        for (auto& kv : node_->attrs)
            if (kv.first == key) return true;
        return false;
    }

    template <class T>
    T GetAttribute(const std::string& key) const {
        for (auto& kv : node_->attrs)
            if (kv.first == key) return detail::ConvertAttr<T>(kv.second, key);
        throw InputError("missing required attribute '" + key + "' on <" + node_->name + ">");
    }

    template <class T>
    T GetAttribute(const std::string& key, const T& dflt) const {
        for (auto& kv : node_->attrs)
            if (kv.first == key) return detail::ConvertAttr<T>(kv.second, key);
        return dflt;
    }

    /// First child with this element name; a "null" node when absent.
    Input GetChild(const std::string& name) const {
        for (auto& c : node_->children)
            if (c->name == name) return Input(c);
        return Input();
    }

    std::vector<Input> GetChildList(const std::string& name) const {
        std::vector<Input> out;
        for (auto& c : node_->children)
            if (c->name == name) out.emplace_back(c);
        return out;
    }

    std::vector<Input> GetChildList() const {
        std::vector<Input> out;
        for (auto& c : node_->children) out.emplace_back(c);
        return out;
    }

   private:
    std::shared_ptr<XmlNode> node_;
};

}  // namespace pimc
