// Scene-description node tree with the reference's JSON semantics:
//   * objects keep key order, arrays keep element order;
//   * every scalar becomes a string value node (floats through std::to_string(float),
//     integers through std::to_string(int), booleans as "true"/"false"),
//     as factory/btrc/factory/node/parser.cpp:38-42 does;
//   * "$include{file}" is spliced textually before parsing (parser.cpp:106-136);
//   * "$reference{a/b/c}" string values are replaced by the referenced node itself, so
//     two references share one node and therefore one created object (parser.cpp:138-…).
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bmath.h"

namespace bt::json {

struct Node;
using NodeP = std::shared_ptr<Node>;

struct Node
{
    enum class Kind { Group, Array, Value };
    Kind kind = Kind::Value;
    std::vector<std::pair<std::string, NodeP>> members;  // Group
    std::vector<NodeP> elems;                            // Array
    std::string str;                                     // Value

    bool is_group() const { return kind == Kind::Group; }
    bool is_array() const { return kind == Kind::Array; }
    bool is_value() const { return kind == Kind::Value; }

    NodeP find(const std::string &key) const;
    NodeP child(const std::string &key) const;  // throws when missing
};

struct ParseError : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

// Parse JSON text (comments allowed). No include or reference processing.
NodeP parse_text(const std::string &text);

// Full scene-file pipeline: read, splice includes (searched in include_dir), parse,
// resolve references.
NodeP parse_scene_file(const std::string &path, const std::string &include_dir);
NodeP parse_scene_text(std::string text, const std::string &include_dir);

// Typed accessors (factory/btrc/factory/node/node.cpp semantics).
float as_float(const NodeP &n);
int as_int(const NodeP &n);
bool as_bool(const NodeP &n);
std::string as_string(const NodeP &n);
V3 as_vec3(const NodeP &n);      // [v], [x,y,z] or scalar
V3 as_spectrum(const NodeP &n);  // same shapes, rgb
float as_degree(const NodeP &n); // {"deg": d} or {"rad": r}, in degrees
float as_radian(const NodeP &n); // {"deg": d} or {"rad": r}, in radians

float float_or(const NodeP &parent, const std::string &key, float def);
int int_or(const NodeP &parent, const std::string &key, int def);
bool bool_or(const NodeP &parent, const std::string &key, bool def);

} // namespace bt::json
