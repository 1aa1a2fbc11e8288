// A small YAML-subset reader for sisi4s input files and cc4s tensor headers.
//
// Covers what those files use: block mappings and sequences (indentation),
// "- key: value" items, flow mappings {a: b, c: d} and flow sequences [a, b],
// single/double-quoted and plain scalars, anchors (&name) and aliases
// (*name), comments, and an optional "---" document marker.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace yl {

struct Node;
using NodeP = std::shared_ptr<Node>;

struct Node {
  enum Kind { Null, Scalar, Seq, Map } kind = Null;
  std::string scalar;
  bool quoted = false;
  std::vector<NodeP> seq;
  std::vector<std::pair<std::string, NodeP>> map;

  bool is_map() const { return kind == Map; }
  bool is_seq() const { return kind == Seq; }
  bool is_scalar() const { return kind == Scalar; }
  // mapping lookup (nullptr if absent)
  NodeP get(const std::string &key) const;
  std::string str() const;
  double as_double() const;
  long long as_int() const;
  bool as_bool() const;
};

struct ParseError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

NodeP parse(const std::string &text);
NodeP parse_file(const std::string &path);

// scalar typing used by the step parser: strict integer, then double
bool scalar_is_int(const std::string &s, long long *v);
bool scalar_is_double(const std::string &s, double *v);

}  // namespace yl
