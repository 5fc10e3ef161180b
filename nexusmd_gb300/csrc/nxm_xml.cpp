#include "nxm_xml.h"

#include <cctype>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

namespace nxm {

const XmlNode *XmlNode::child(const char *n) const {
    for (auto &c : children)
        if (c->name == n) return c.get();
    return nullptr;
}

std::vector<const XmlNode *> XmlNode::children_named(const char *n) const {
    std::vector<const XmlNode *> out;
    for (auto &c : children)
        if (c->name == n) out.push_back(c.get());
    return out;
}

const char *XmlNode::attr(const char *n) const {
    for (auto &a : attrs)
        if (a.first == n) return a.second.c_str();
    return nullptr;
}

double XmlNode::as_double(const char *n) const {
    const char *v = attr(n);
    if (!v) return 0.0;
    return std::strtod(v, nullptr);
}

int XmlNode::as_int(const char *n) const {
    const char *v = attr(n);
    if (!v) return 0;
    return (int)std::strtol(v, nullptr, 0);
}

namespace {

struct Parser {
    const std::string &s;
    size_t p = 0;
    std::string err;

    explicit Parser(const std::string &t) : s(t) {}

    bool fail(const char *why) {
        if (err.empty()) {
            std::ostringstream o;
            o << why << " at offset " << p;
            err = o.str();
        }
        return false;
    }
    static bool space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }
    void skip_ws() {
        while (p < s.size() && space(s[p])) ++p;
    }
    bool starts(const char *t) const { return s.compare(p, std::strlen(t), t) == 0; }
    bool skip_until(const char *t) {
        size_t q = s.find(t, p);
        if (q == std::string::npos) return fail("unterminated construct");
        p = q + std::strlen(t);
        return true;
    }
    static bool name_char(char c) {
        return std::isalnum((unsigned char)c) || c == '_' || c == ':' || c == '-' || c == '.';
    }
    std::string name() {
        size_t q = p;
        while (p < s.size() && name_char(s[p])) ++p;
        return s.substr(q, p - q);
    }
    static std::string decode(const std::string &v) {
        if (v.find('&') == std::string::npos) return v;
        std::string o;
        for (size_t i = 0; i < v.size(); ++i) {
            if (v[i] != '&') {
                o += v[i];
                continue;
            }
            static const char *ent[5][2] = {{"&lt;", "<"}, {"&gt;", ">"}, {"&amp;", "&"}, {"&quot;", "\""}, {"&apos;", "'"}};
            bool done = false;
            for (auto &e : ent)
                if (v.compare(i, std::strlen(e[0]), e[0]) == 0) {
                    o += e[1];
                    i += std::strlen(e[0]) - 1;
                    done = true;
                    break;
                }
            if (!done) o += '&';
        }
        return o;
    }
    // skip text, comments, processing instructions and doctype until '<' of an element or a close tag
    bool misc() {
        for (;;) {
            while (p < s.size() && s[p] != '<') ++p;
            if (p >= s.size()) return true;
            if (starts("<!--")) {
                if (!skip_until("-->")) return false;
            } else if (starts("<?")) {
                if (!skip_until("?>")) return false;
            } else if (starts("<![CDATA[")) {
                if (!skip_until("]]>")) return false;
            } else if (starts("<!")) {
                if (!skip_until(">")) return false;
            } else {
                return true;
            }
        }
    }
    bool element(XmlNode &parent) {
        // at '<' of a start tag
        ++p;
        auto node = std::make_unique<XmlNode>();
        node->name = name();
        if (node->name.empty()) return fail("missing element name");
        for (;;) {
            skip_ws();
            if (p >= s.size()) return fail("unterminated start tag");
            if (s[p] == '/') {
                if (p + 1 >= s.size() || s[p + 1] != '>') return fail("bad self-closing tag");
                p += 2;
                parent.children.push_back(std::move(node));
                return true;
            }
            if (s[p] == '>') {
                ++p;
                break;
            }
            std::string an = name();
            if (an.empty()) return fail("bad attribute name");
            skip_ws();
            if (p >= s.size() || s[p] != '=') return fail("expected '='");
            ++p;
            skip_ws();
            if (p >= s.size() || (s[p] != '"' && s[p] != '\'')) return fail("expected quoted value");
            char qch = s[p++];
            size_t q = s.find(qch, p);
            if (q == std::string::npos) return fail("unterminated attribute value");
            node->attrs.emplace_back(an, decode(s.substr(p, q - p)));
            p = q + 1;
        }
        // content
        for (;;) {
            if (!misc()) return false;
            if (p >= s.size()) return fail("missing end tag");
            if (starts("</")) {
                p += 2;
                std::string en = name();
                if (en != node->name) return fail("mismatched end tag");
                skip_ws();
                if (p >= s.size() || s[p] != '>') return fail("bad end tag");
                ++p;
                parent.children.push_back(std::move(node));
                return true;
            }
            if (!element(*node)) return false;
        }
    }
    bool document(XmlNode &root) {
        for (;;) {
            if (!misc()) return false;
            if (p >= s.size()) break;
            if (starts("</")) return fail("unexpected end tag");
            if (!element(root)) return false;
        }
        if (root.children.empty()) return fail("no document element");
        return true;
    }
};

}  // namespace

XmlDoc xml_parse(const std::string &text) {
    XmlDoc d;
    Parser ps(text);
    if (!ps.document(d.root)) d.error = ps.err;
    return d;
}

XmlDoc xml_load_file(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) {
        XmlDoc d;
        d.error = "File was not found";
        return d;
    }
    std::ostringstream o;
    o << f.rdbuf();
    return xml_parse(o.str());
}

}  // namespace nxm
