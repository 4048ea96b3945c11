// yaml_lite.h -- the YAML subset SHAW input files use (yaml-cpp is not available):
// block mappings, block sequences ("- x", also at the parent key's indent),
// flow mappings "{a: 1, b: [1, 2]}", flow sequences, plain/quoted scalars and
// '#' comments.  Values are kept as strings and converted on access with the
// same acceptance rules the reference's yaml-cpp calls rely on.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace shaw {
namespace yaml {

struct Node {
  enum Kind { Null, Scalar, Seq, Map } kind = Null;
  std::string scalar;
  std::vector<Node> seq;
  std::vector<std::pair<std::string, Node>> map;

  bool is_null() const { return kind == Null; }
  bool is_scalar() const { return kind == Scalar; }
  bool is_seq() const { return kind == Seq; }
  bool is_map() const { return kind == Map; }
  // Returns nullptr when the key is absent (yaml-cpp: an undefined node).
  const Node* get(const std::string& key) const;

  std::string as_string() const;
  double as_double() const;
  bool as_bool() const;
  long long as_int() const;
  unsigned long long as_size() const;
  std::vector<double> as_double_vector() const;
};

// Throws std::runtime_error on syntax errors or a missing file.
Node parse_file(const std::string& path);
Node parse_string(const std::string& text);

}  // namespace yaml
}  // namespace shaw
