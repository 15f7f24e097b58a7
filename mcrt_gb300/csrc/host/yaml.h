// yaml.h — a small YAML reader for the scene format (block mappings, block
// sequences, flow [..] and {..} collections, plain/quoted scalars, comments).
// The reference parses scenes with serde_yml 0.0.12 (src/scene.rs:645); this
// reader covers the subset the scene files use and reports anything else
// (anchors, tags, multi-line scalars, documents) as a parse error.
#pragma once

#include <string>
#include <utility>
#include <vector>

namespace mcrt_host {

struct YNode {
    enum Kind { Null, Scalar, Map, Seq } kind = Null;
    std::string scalar;
    bool quoted = false;
    std::vector<std::pair<std::string, YNode>> map;
    std::vector<YNode> seq;
    int line = 0;

    const YNode *get(const std::string &key) const {
        for (const auto &kv : map)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

// Parse `text`; on failure returns false and sets *err ("line N: ...").
bool yaml_parse(const std::string &text, YNode *out, std::string *err);

}  // namespace mcrt_host
