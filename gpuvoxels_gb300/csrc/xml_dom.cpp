#include "xml_dom.h"

#include <cctype>
#include <cstring>

namespace gvx {

const XmlNode* XmlNode::child(const std::string& name) const {
    for (auto& c : children)
        if (c->tag == name) return c.get();
    return nullptr;
}
XmlNode* XmlNode::child(const std::string& name) {
    for (auto& c : children)
        if (c->tag == name) return c.get();
    return nullptr;
}
std::vector<const XmlNode*> XmlNode::children_named(const std::string& name) const {
    std::vector<const XmlNode*> r;
    for (auto& c : children)
        if (c->tag == name) r.push_back(c.get());
    return r;
}
const char* XmlNode::attr(const std::string& name) const {
    for (auto& a : attrs)
        if (a.first == name) return a.second.c_str();
    return nullptr;
}
const XmlNode* XmlNode::path(const std::string& dotted) const {
    size_t start = 0;
    const XmlNode* node = nullptr;
    while (start <= dotted.size()) {
        size_t dot = dotted.find('.', start);
        std::string part = dotted.substr(start, dot == std::string::npos ? std::string::npos : dot - start);
        if (!node) {
            if (part != tag) return nullptr;
            node = this;
        } else {
            node = node->child(part);
            if (!node) return nullptr;
        }
        if (dot == std::string::npos) break;
        start = dot + 1;
    }
    return node;
}
std::unique_ptr<XmlNode> XmlNode::clone() const {
    auto n = std::make_unique<XmlNode>();
    n->tag = tag;
    n->attrs = attrs;
    n->text = text;
    for (auto& c : children) n->children.push_back(c->clone());
    return n;
}

namespace {
struct Parser {
    const std::string& s;
    size_t i = 0;
    std::string err;
    explicit Parser(const std::string& src) : s(src) {}

    bool starts(const char* p) const { return s.compare(i, strlen(p), p) == 0; }
    void skip_ws() { while (i < s.size() && isspace((unsigned char)s[i])) i++; }
    bool fail(const std::string& m) { if (err.empty()) err = m + " at offset " + std::to_string(i); return false; }

    // appends the text s[b, e) to out with its entity references replaced
    void decode_into(size_t b, size_t e, std::string* out) const {
        const char* amp = (const char*)memchr(s.data() + b, '&', e - b);
        if (!amp) { out->append(s, b, e - b); return; }   // the usual case: no references
        const std::string in = s.substr(b, e - b);
        out->reserve(out->size() + in.size());
        for (size_t k = 0; k < in.size(); k++) {
            if (in[k] != '&') { *out += in[k]; continue; }
            size_t semi = in.find(';', k);
            if (semi == std::string::npos) { *out += in[k]; continue; }
            std::string ent = in.substr(k + 1, semi - k - 1);
            if (ent == "lt") *out += '<';
            else if (ent == "gt") *out += '>';
            else if (ent == "amp") *out += '&';
            else if (ent == "quot") *out += '"';
            else if (ent == "apos") *out += '\'';
            else if (!ent.empty() && ent[0] == '#') {
                long code = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X') ? strtol(ent.c_str() + 2, nullptr, 16) : strtol(ent.c_str() + 1, nullptr, 10);
                if (code > 0 && code < 128) *out += (char)code;
            } else { *out += '&'; continue; }
            k = semi;
        }
    }
    bool skip_misc() {  // comments, declarations, processing instructions
        for (;;) {
            skip_ws();
            if (starts("<?")) {
                size_t e = s.find("?>", i);
                if (e == std::string::npos) return fail("unterminated processing instruction");
                i = e + 2;
            } else if (starts("<!--")) {
                size_t e = s.find("-->", i);
                if (e == std::string::npos) return fail("unterminated comment");
                i = e + 3;
            } else if (starts("<!DOCTYPE")) {
                size_t e = s.find('>', i);
                if (e == std::string::npos) return fail("unterminated doctype");
                i = e + 1;
            } else return true;
        }
    }
    bool name(std::string* out) {
        size_t b = i;
        while (i < s.size() && (isalnum((unsigned char)s[i]) || s[i] == '_' || s[i] == '-' || s[i] == ':' || s[i] == '.')) i++;
        if (i == b) return fail("expected a name");
        out->assign(s, b, i - b);
        return true;
    }
    bool element(XmlNode* n, int depth) {
        if (depth > 200) return fail("nesting too deep");
        if (i >= s.size() || s[i] != '<') return fail("expected '<'");
        i++;
        if (!name(&n->tag)) return false;
        for (;;) {
            skip_ws();
            if (i >= s.size()) return fail("unexpected end in tag");
            if (s[i] == '/') {
                if (i + 1 < s.size() && s[i + 1] == '>') { i += 2; return true; }
                return fail("bad '/' in tag");
            }
            if (s[i] == '>') { i++; break; }
            std::string an;
            if (!name(&an)) return false;
            skip_ws();
            if (i >= s.size() || s[i] != '=') return fail("expected '=' after attribute");
            i++;
            skip_ws();
            if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) return fail("expected quoted attribute");
            char q = s[i++];
            size_t e = s.find(q, i);
            if (e == std::string::npos) return fail("unterminated attribute");
            n->attrs.emplace_back(std::move(an), std::string());
            decode_into(i, e, &n->attrs.back().second);
            i = e + 1;
        }
        for (;;) {
            if (i >= s.size()) return fail("unterminated element <" + n->tag + ">");
            if (starts("</")) {
                i += 2;
                std::string close;
                if (!name(&close)) return false;
                if (close != n->tag) return fail("mismatched </" + close + "> for <" + n->tag + ">");
                skip_ws();
                if (i >= s.size() || s[i] != '>') return fail("expected '>'");
                i++;
                return true;
            } else if (starts("<![CDATA[")) {
                size_t e = s.find("]]>", i);
                if (e == std::string::npos) return fail("unterminated CDATA");
                n->text.append(s, i + 9, e - i - 9);
                i = e + 3;
            } else if (starts("<!--")) {
                size_t e = s.find("-->", i);
                if (e == std::string::npos) return fail("unterminated comment");
                i = e + 3;
            } else if (starts("<?")) {
                size_t e = s.find("?>", i);
                if (e == std::string::npos) return fail("unterminated processing instruction");
                i = e + 2;
            } else if (s[i] == '<') {
                auto c = std::make_unique<XmlNode>();
                if (!element(c.get(), depth + 1)) return false;
                n->children.push_back(std::move(c));
            } else {
                size_t e = s.find('<', i);
                if (e == std::string::npos) e = s.size();
                decode_into(i, e, &n->text);
                i = e;
            }
        }
    }
};
}  // namespace

std::unique_ptr<XmlNode> xml_parse(const std::string& src, std::string* err) {
    Parser p(src);
    auto root = std::make_unique<XmlNode>();
    if (!p.skip_misc() || !p.element(root.get(), 0)) {
        if (err) *err = p.err.empty() ? "malformed XML" : p.err;
        return nullptr;
    }
    return root;
}

std::string xml_escape(const std::string& in) {
    std::string o;
    for (char c : in) {
        if (c == '<') o += "&lt;";
        else if (c == '>') o += "&gt;";
        else if (c == '&') o += "&amp;";
        else if (c == '"') o += "&quot;";
        else o += c;
    }
    return o;
}

std::string xml_write(const XmlNode& n, int indent) {
    std::string pad(indent * 2, ' ');
    std::string o = pad + "<" + n.tag;
    for (auto& a : n.attrs) o += " " + a.first + "=\"" + xml_escape(a.second) + "\"";
    if (n.children.empty()) {
        if (n.text.empty()) return o + "/>\n";
        return o + ">" + xml_escape(n.text) + "</" + n.tag + ">\n";
    }
    o += ">\n";
    for (auto& c : n.children) o += xml_write(*c, indent + 1);
    return o + pad + "</" + n.tag + ">\n";
}

}  // namespace gvx
