#include "xml.hpp"
#include "error.hpp"
#include <fstream>
#include <sstream>
#include <cstring>
#include <cctype>

namespace spn {

const std::string *XmlNode::attr(const std::string &key) const {
    for (auto &a : attrs)
        if (a.first == key) return &a.second;
    return nullptr;
}

const XmlNode *XmlNode::child(const std::string &key) const {
    for (auto &c : children)
        if (c.name == key) return &c;
    return nullptr;
}

int XmlNode::count(const std::string &key) const {
    int n = 0;
    for (auto &c : children) n += (c.name == key);
    return n;
}

namespace {

struct Cursor {
    const std::string &s;
    size_t i = 0;
    explicit Cursor(const std::string &str) : s(str) {}
    bool eof() const { return i >= s.size(); }
    bool starts(const char *p) const { return s.compare(i, std::strlen(p), p) == 0; }
    [[noreturn]] void fail(const std::string &what) const {
        throw Error(ErrorType::Initialization, "XML parse error at offset " + std::to_string(i) + ": " + what);
    }
    void skip_ws() {
        while (!eof() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r' || s[i] == '\n')) ++i;
    }
    void skip_until(const char *end) {
        size_t p = s.find(end, i);
        if (p == std::string::npos) fail(std::string("unterminated construct, expected ") + end);
        i = p + std::strlen(end);
    }
};

std::string decode_entities(const std::string &in) {
    std::string out;
    out.reserve(in.size());
    for (size_t i = 0; i < in.size(); ++i) {
        if (in[i] != '&') {
            out += in[i];
            continue;
        }
        size_t semi = in.find(';', i);
        if (semi == std::string::npos) {
            out += in[i];
            continue;
        }
        std::string ent = in.substr(i + 1, semi - i - 1);
        if (ent == "lt") out += '<';
        else if (ent == "gt") out += '>';
        else if (ent == "amp") out += '&';
        else if (ent == "quot") out += '"';
        else if (ent == "apos") out += '\'';
        else if (!ent.empty() && ent[0] == '#') {
            long code = (ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X')) ? std::strtol(ent.c_str() + 2, nullptr, 16)
                                                                              : std::strtol(ent.c_str() + 1, nullptr, 10);
            if (code > 0 && code < 128) out += char(code);
        } else {
            out += in.substr(i, semi - i + 1);
        }
        i = semi;
    }
    return out;
}

bool is_name_char(char c) {
    return std::isalnum(static_cast<unsigned char>(c)) || c == '_' || c == '-' || c == '.' || c == ':';
}

std::string parse_name(Cursor &c) {
    size_t b = c.i;
    while (!c.eof() && is_name_char(c.s[c.i])) ++c.i;
    if (b == c.i) c.fail("expected a name");
    return c.s.substr(b, c.i - b);
}

// Skips comments, processing instructions, doctype and whitespace between elements.
void skip_misc(Cursor &c) {
    for (;;) {
        c.skip_ws();
        if (c.starts("<!--")) c.skip_until("-->");
        else if (c.starts("<?")) c.skip_until("?>");
        else if (c.starts("<!DOCTYPE")) c.skip_until(">");
        else return;
    }
}

XmlNode parse_element(Cursor &c, int depth) {
    if (depth > 256) c.fail("nesting too deep");
    if (c.eof() || c.s[c.i] != '<') c.fail("expected '<'");
    ++c.i;
    XmlNode node;
    node.name = parse_name(c);
    for (;;) {
        c.skip_ws();
        if (c.eof()) c.fail("unterminated start tag");
        if (c.starts("/>")) {
            c.i += 2;
            return node;
        }
        if (c.s[c.i] == '>') {
            ++c.i;
            break;
        }
        std::string key = parse_name(c);
        c.skip_ws();
        if (c.eof() || c.s[c.i] != '=') c.fail("expected '=' after attribute " + key);
        ++c.i;
        c.skip_ws();
        if (c.eof() || (c.s[c.i] != '"' && c.s[c.i] != '\'')) c.fail("expected quoted attribute value");
        char q = c.s[c.i++];
        size_t e = c.s.find(q, c.i);
        if (e == std::string::npos) c.fail("unterminated attribute value");
        node.attrs.emplace_back(key, decode_entities(c.s.substr(c.i, e - c.i)));
        c.i = e + 1;
    }
    // content
    for (;;) {
        if (c.eof()) c.fail("unterminated element <" + node.name + ">");
        if (c.starts("</")) {
            c.i += 2;
            std::string close = parse_name(c);
            if (close != node.name) c.fail("mismatched closing tag </" + close + "> for <" + node.name + ">");
            c.skip_ws();
            if (c.eof() || c.s[c.i] != '>') c.fail("expected '>'");
            ++c.i;
            return node;
        }
        if (c.starts("<!--")) {
            c.skip_until("-->");
            continue;
        }
        if (c.starts("<![CDATA[")) {
            size_t b = c.i + 9;
            c.skip_until("]]>");
            node.text += c.s.substr(b, c.i - 3 - b);
            continue;
        }
        if (c.starts("<?")) {
            c.skip_until("?>");
            continue;
        }
        if (c.s[c.i] == '<') {
            node.children.push_back(parse_element(c, depth + 1));
            continue;
        }
        size_t e = c.s.find('<', c.i);
        if (e == std::string::npos) e = c.s.size();
        std::string raw = c.s.substr(c.i, e - c.i);
        // whitespace-only runs between child elements are not text
        if (raw.find_first_not_of(" \t\r\n") != std::string::npos) node.text += decode_entities(raw);
        c.i = e;
    }
}

void serialize(const XmlNode &n, int indent, std::ostringstream &os) {
    std::string pad(indent * 4, ' ');
    os << pad << '<' << n.name;
    for (auto &a : n.attrs) os << ' ' << a.first << "=\"" << a.second << '"';
    if (n.children.empty() && n.text.empty()) {
        os << "/>\n";
        return;
    }
    os << '>';
    if (n.children.empty()) {
        os << n.text << "</" << n.name << ">\n";
        return;
    }
    os << '\n';
    for (auto &ch : n.children) serialize(ch, indent + 1, os);
    os << pad << "</" << n.name << ">\n";
}

}  // namespace

XmlNode xml_parse_string(const std::string &doc) {
    Cursor c(doc);
    XmlNode root;
    root.name = "";
    for (;;) {
        skip_misc(c);
        if (c.eof()) break;
        root.children.push_back(parse_element(c, 0));
    }
    return root;
}

XmlNode xml_parse_file(const std::string &path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw Error(ErrorType::IO, "cannot open XML file '" + path + "'");
    std::stringstream ss;
    ss << f.rdbuf();
    return xml_parse_string(ss.str());
}

std::string xml_serialize(const XmlNode &root) {
    std::ostringstream os;
    os << "<?xml version=\"1.0\" encoding=\"utf-8\"?>\n";
    for (auto &c : root.children) serialize(c, 0, os);
    return os.str();
}

}  // namespace spn
