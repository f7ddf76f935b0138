// xml.cpp -- recursive-descent XML reader (see xml.h).
#include "xml.h"

#include <cctype>

namespace Pupil::xml {

const std::string *Node::attr(const std::string &key) const {
    for (auto &kv : attrs)
        if (kv.first == key) return &kv.second;
    return nullptr;
}

std::string Node::attr_or(const std::string &key, const std::string &fallback) const {
    const std::string *v = attr(key);
    return v ? *v : fallback;
}

namespace {

struct Reader {
    const std::string &s;
    size_t i = 0;
    int line = 1;
    std::string err;

    bool eof() const { return i >= s.size(); }
    char peek(size_t k = 0) const { return i + k < s.size() ? s[i + k] : '\0'; }
    void adv(size_t n = 1) {
        for (size_t k = 0; k < n && i < s.size(); k++, i++)
            if (s[i] == '\n') line++;
    }
    bool starts(const char *lit) const { return s.compare(i, std::char_traits<char>::length(lit), lit) == 0; }
    void ws() {
        while (!eof() && std::isspace(static_cast<unsigned char>(peek()))) adv();
    }
    bool fail(const std::string &m) {
        if (err.empty()) err = "line " + std::to_string(line) + ": " + m;
        return false;
    }
    bool skip_until(const char *lit) {
        size_t p = s.find(lit, i);
        if (p == std::string::npos) return fail(std::string("unterminated construct, expected ") + lit);
        adv(p - i + std::char_traits<char>::length(lit));
        return true;
    }
    // comments, processing instructions and DOCTYPE between elements
    bool misc() {
        for (;;) {
            ws();
            if (starts("<!--")) {
                if (!skip_until("-->")) return false;
            } else if (starts("<?")) {
                if (!skip_until("?>")) return false;
            } else if (starts("<!")) {
                if (!skip_until(">")) return false;
            } else {
                return true;
            }
        }
    }
    bool name(std::string &out) {
        size_t b = i;
        while (!eof() && (std::isalnum(static_cast<unsigned char>(peek())) || peek() == '_' || peek() == '-' ||
                          peek() == ':' || peek() == '.'))
            adv();
        if (i == b) return fail("expected a name");
        out = s.substr(b, i - b);
        return true;
    }
    static void unescape(std::string &v) {
        static const std::pair<const char *, char> ents[] = {{"&lt;", '<'}, {"&gt;", '>'}, {"&quot;", '"'},
                                                             {"&apos;", '\''}, {"&amp;", '&'}};
        for (auto &e : ents) {
            size_t p = 0;
            std::string key = e.first;
            while ((p = v.find(key, p)) != std::string::npos) {
                v.replace(p, key.size(), 1, e.second);
                p += 1;
            }
        }
    }
    std::unique_ptr<Node> element(int depth) {
        if (depth > 256) {
            fail("nesting too deep");
            return nullptr;
        }
        if (peek() != '<') {
            fail("expected '<'");
            return nullptr;
        }
        adv();
        auto n = std::make_unique<Node>();
        n->line = line;
        if (!name(n->name)) return nullptr;
        for (;;) {
            ws();
            if (starts("/>")) {
                adv(2);
                return n;
            }
            if (peek() == '>') {
                adv();
                break;
            }
            std::string key;
            if (!name(key)) return nullptr;
            ws();
            if (peek() != '=') {
                fail("expected '=' after attribute " + key);
                return nullptr;
            }
            adv();
            ws();
            char q = peek();
            if (q != '"' && q != '\'') {
                fail("expected a quoted value for attribute " + key);
                return nullptr;
            }
            adv();
            size_t e = s.find(q, i);
            if (e == std::string::npos) {
                fail("unterminated attribute value");
                return nullptr;
            }
            std::string v = s.substr(i, e - i);
            adv(e - i + 1);
            unescape(v);
            n->attrs.emplace_back(std::move(key), std::move(v));
        }
        for (;;) {
            if (!misc()) return nullptr;
            if (eof()) {
                fail("unexpected end of file inside <" + n->name + ">");
                return nullptr;
            }
            if (starts("</")) {
                adv(2);
                std::string close;
                if (!name(close)) return nullptr;
                if (close != n->name) {
                    fail("mismatched </" + close + "> for <" + n->name + ">");
                    return nullptr;
                }
                ws();
                if (peek() != '>') {
                    fail("expected '>'");
                    return nullptr;
                }
                adv();
                return n;
            }
            if (peek() == '<') {
                auto c = element(depth + 1);
                if (!c) return nullptr;
                n->children.push_back(std::move(c));
            } else {
                while (!eof() && peek() != '<') adv();  // character data is not used by the format
            }
        }
    }
};

}  // namespace

std::unique_ptr<Node> Parse(const std::string &text, std::string &error) {
    Reader r{text};
    if (!r.misc()) {
        error = r.err;
        return nullptr;
    }
    auto root = r.element(0);
    if (!root) {
        error = r.err.empty() ? "malformed document" : r.err;
        return nullptr;
    }
    if (!r.misc()) {
        error = r.err;
        return nullptr;
    }
    r.ws();
    if (!r.eof()) {
        error = "line " + std::to_string(r.line) + ": content after the root element";
        return nullptr;
    }
    return root;
}

}  // namespace Pupil::xml
