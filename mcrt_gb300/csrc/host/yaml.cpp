// yaml.cpp — see yaml.h.
#include "yaml.h"

#include <cstring>

namespace mcrt_host {

namespace {

struct Line {
    int indent;
    std::string text;   // without indentation and comment
    int number;         // 1-based
};

// Strip a comment: '#' at the start or preceded by whitespace, outside quotes.
std::string strip_comment(const std::string &s) {
    char q = 0;
    for (size_t i = 0; i < s.size(); ++i) {
        char c = s[i];
        if (q) {
            if (c == q) q = 0;
            continue;
        }
        if (c == '\'' || c == '"') q = c;
        else if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) return s.substr(0, i);
    }
    return s;
}

std::string rtrim(const std::string &s) {
    size_t e = s.size();
    while (e > 0 && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\r')) --e;
    return s.substr(0, e);
}
std::string trim(const std::string &s) {
    size_t b = 0;
    while (b < s.size() && (s[b] == ' ' || s[b] == '\t')) ++b;
    return rtrim(s.substr(b));
}

struct Parser {
    std::vector<Line> lines;
    std::string err;

    bool fail(int line, const std::string &m) {
        if (err.empty()) err = "line " + std::to_string(line) + ": " + m;
        return false;
    }

    // ---- flow / scalar parsing over a single string
    bool parse_flow(const std::string &s, size_t &i, YNode *out, int line, bool in_flow) {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
        out->line = line;
        if (i >= s.size()) { out->kind = YNode::Null; return true; }
        char c = s[i];
        if (c == '[') {
            out->kind = YNode::Seq;
            ++i;
            for (;;) {
                while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
                if (i >= s.size()) return fail(line, "unterminated '['");
                if (s[i] == ']') { ++i; return true; }
                YNode item;
                if (!parse_flow(s, i, &item, line, true)) return false;
                out->seq.push_back(item);
                while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
                if (i < s.size() && s[i] == ',') { ++i; continue; }
                if (i < s.size() && s[i] == ']') { ++i; return true; }
                return fail(line, "expected ',' or ']' in flow sequence");
            }
        }
        if (c == '{') {
            out->kind = YNode::Map;
            ++i;
            for (;;) {
                while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
                if (i >= s.size()) return fail(line, "unterminated '{'");
                if (s[i] == '}') { ++i; return true; }
                YNode key;
                if (!parse_scalar(s, i, &key, line, true, true)) return false;
                while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
                if (i >= s.size() || s[i] != ':') return fail(line, "expected ':' in flow mapping");
                ++i;
                YNode val;
                if (!parse_flow(s, i, &val, line, true)) return false;
                if (out->get(key.scalar)) return fail(line, "duplicate key '" + key.scalar + "'");
                out->map.push_back({key.scalar, val});
                while (i < s.size() && (s[i] == ' ' || s[i] == '\t')) ++i;
                if (i < s.size() && s[i] == ',') { ++i; continue; }
                if (i < s.size() && s[i] == '}') { ++i; return true; }
                return fail(line, "expected ',' or '}' in flow mapping");
            }
        }
        return parse_scalar(s, i, out, line, in_flow, false);
    }

    bool parse_scalar(const std::string &s, size_t &i, YNode *out, int line, bool in_flow, bool is_key) {
        out->kind = YNode::Scalar;
        out->line = line;
        if (i < s.size() && (s[i] == '"' || s[i] == '\'')) {
            char q = s[i++];
            std::string v;
            while (i < s.size() && s[i] != q) {
                if (q == '"' && s[i] == '\\' && i + 1 < s.size()) {
                    char e = s[i + 1];
                    v += e == 'n' ? '\n' : e == 't' ? '\t' : e;
                    i += 2;
                    continue;
                }
                if (q == '\'' && s[i] == '\'' && i + 1 < s.size() && s[i + 1] == '\'') { v += '\''; i += 2; continue; }
                v += s[i++];
            }
            if (i >= s.size()) return fail(line, "unterminated quoted scalar");
            ++i;
            out->scalar = v;
            out->quoted = true;
            return true;
        }
        size_t b = i;
        while (i < s.size()) {
            char c = s[i];
            if (in_flow && (c == ',' || c == ']' || c == '}')) break;
            if (is_key && c == ':') break;
            ++i;
        }
        out->scalar = trim(s.substr(b, i - b));
        if (!is_key && out->scalar.empty()) out->kind = YNode::Null;
        if (!out->scalar.empty() && (out->scalar[0] == '&' || out->scalar[0] == '*' || out->scalar[0] == '!' ||
                                     out->scalar[0] == '|' || out->scalar[0] == '>'))
            return fail(line, "unsupported YAML construct '" + out->scalar.substr(0, 1) + "'");
        if (!is_key && out->scalar == "~") out->kind = YNode::Null;
        if (!is_key && (out->scalar == "null" || out->scalar == "Null")) out->kind = YNode::Null;
        return true;
    }

    // Flow collections may continue over following lines until brackets balance.
    std::string gather_flow(size_t &li, const std::string &first) {
        std::string acc = first;
        auto depth = [](const std::string &s) {
            int d = 0;
            char q = 0;
            for (char c : s) {
                if (q) { if (c == q) q = 0; continue; }
                if (c == '"' || c == '\'') q = c;
                else if (c == '[' || c == '{') ++d;
                else if (c == ']' || c == '}') --d;
            }
            return d;
        };
        while (depth(acc) > 0 && li + 1 < lines.size()) {
            ++li;
            acc += " " + lines[li].text;
        }
        return acc;
    }

    // Split "key: rest" at the first ':' followed by space/end outside quotes and brackets.
    static bool split_key(const std::string &t, std::string *key, std::string *rest) {
        char q = 0;
        int d = 0;
        for (size_t i = 0; i < t.size(); ++i) {
            char c = t[i];
            if (q) { if (c == q) q = 0; continue; }
            if (c == '"' || c == '\'') q = c;
            else if (c == '[' || c == '{') ++d;
            else if (c == ']' || c == '}') --d;
            else if (c == ':' && d == 0 && (i + 1 == t.size() || t[i + 1] == ' ' || t[i + 1] == '\t')) {
                *key = trim(t.substr(0, i));
                *rest = trim(t.substr(i + 1));
                if (key->size() >= 2 && (((*key)[0] == '"' && key->back() == '"') ||
                                         ((*key)[0] == '\'' && key->back() == '\'')))
                    *key = key->substr(1, key->size() - 2);
                return true;
            }
        }
        return false;
    }

    bool parse_value_text(size_t &li, const std::string &text, YNode *out) {
        std::string full = text;
        if (!text.empty() && (text[0] == '[' || text[0] == '{')) full = gather_flow(li, text);
        size_t i = 0;
        if (!parse_flow(full, i, out, lines[li].number, false)) return false;
        while (i < full.size() && (full[i] == ' ' || full[i] == '\t')) ++i;
        if (i != full.size()) return fail(lines[li].number, "unexpected text after value");
        return true;
    }

    // Parse the block starting at line li with indentation `indent`.
    bool parse_block(size_t &li, int indent, YNode *out) {
        if (li >= lines.size()) { out->kind = YNode::Null; return true; }
        const bool is_seq = lines[li].text.size() >= 1 && lines[li].text[0] == '-' &&
                            (lines[li].text.size() == 1 || lines[li].text[1] == ' ');
        out->line = lines[li].number;
        if (is_seq) {
            out->kind = YNode::Seq;
            while (li < lines.size() && lines[li].indent == indent && !lines[li].text.empty() &&
                   lines[li].text[0] == '-' && (lines[li].text.size() == 1 || lines[li].text[1] == ' ')) {
                std::string rest = lines[li].text.size() > 1 ? lines[li].text.substr(2) : "";
                size_t pad = 2;
                while (pad < lines[li].text.size() && lines[li].text[pad] == ' ') ++pad;
                rest = trim(rest);
                YNode item;
                if (rest.empty()) {
                    ++li;
                    if (li < lines.size() && lines[li].indent > indent) {
                        if (!parse_block(li, lines[li].indent, &item)) return false;
                    } else {
                        item.kind = YNode::Null;
                    }
                } else {
                    std::string k, r;
                    if (rest[0] != '[' && rest[0] != '{' && rest[0] != '"' && rest[0] != '\'' && split_key(rest, &k, &r)) {
                        // "- key: value ..." starts a mapping at the column of `key`
                        lines[li].indent = indent + (int)pad;
                        lines[li].text = rest;
                        if (!parse_block(li, indent + (int)pad, &item)) return false;
                    } else {
                        if (!parse_value_text(li, rest, &item)) return false;
                        ++li;
                    }
                }
                out->seq.push_back(item);
            }
            if (li < lines.size() && lines[li].indent > indent)
                return fail(lines[li].number, "bad indentation in sequence");
            return true;
        }
        out->kind = YNode::Map;
        while (li < lines.size() && lines[li].indent == indent) {
            const Line &ln = lines[li];
            if (!ln.text.empty() && ln.text[0] == '-') return fail(ln.number, "sequence item inside a mapping");
            std::string key, rest;
            if (!split_key(ln.text, &key, &rest)) return fail(ln.number, "expected 'key: value'");
            if (out->get(key)) return fail(ln.number, "duplicate key '" + key + "'");
            YNode val;
            if (rest.empty()) {
                ++li;
                if (li < lines.size() && lines[li].indent > indent) {
                    if (!parse_block(li, lines[li].indent, &val)) return false;
                } else if (li < lines.size() && lines[li].indent == indent && lines[li].text[0] == '-' &&
                           (lines[li].text.size() == 1 || lines[li].text[1] == ' ')) {
                    if (!parse_block(li, indent, &val)) return false;   // "key:\n- item" at the same indent
                } else {
                    val.kind = YNode::Null;
                    val.line = ln.number;
                }
            } else {
                if (!parse_value_text(li, rest, &val)) return false;
                ++li;
            }
            out->map.push_back({key, val});
        }
        if (li < lines.size() && lines[li].indent > indent) return fail(lines[li].number, "bad indentation");
        return true;
    }
};

}  // namespace

bool yaml_parse(const std::string &text, YNode *out, std::string *err) {
    Parser p;
    size_t pos = 0;
    int number = 0;
    while (pos <= text.size()) {
        size_t nl = text.find('\n', pos);
        std::string raw = text.substr(pos, nl == std::string::npos ? std::string::npos : nl - pos);
        ++number;
        pos = nl == std::string::npos ? text.size() + 1 : nl + 1;
        if (raw.find('\t') != std::string::npos) {
            size_t ind = raw.find_first_not_of(' ');
            if (ind != std::string::npos && raw[ind] == '\t') {
                if (err) *err = "line " + std::to_string(number) + ": tab indentation";
                return false;
            }
        }
        std::string s = rtrim(strip_comment(raw));
        size_t ind = s.find_first_not_of(' ');
        if (ind == std::string::npos) continue;
        std::string body = s.substr(ind);
        if (body == "---" || body == "...") {
            if (p.lines.empty() && body == "---") continue;
            if (err) *err = "line " + std::to_string(number) + ": multiple documents are not supported";
            return false;
        }
        p.lines.push_back({(int)ind, body, number});
    }
    *out = YNode();
    if (p.lines.empty()) { out->kind = YNode::Map; return true; }
    size_t li = 0;
    if (p.lines[0].indent != 0) {
        if (err) *err = "line " + std::to_string(p.lines[0].number) + ": top level must not be indented";
        return false;
    }
    if (!p.parse_block(li, 0, out)) {
        if (err) *err = p.err;
        return false;
    }
    if (li != p.lines.size()) {
        if (err) *err = "line " + std::to_string(p.lines[li].number) + ": unexpected content";
        return false;
    }
    return true;
}

}  // namespace mcrt_host
