// Reader for the HSD input subset the fnet program takes (fortnet_in.hsd): nested blocks
// `Key { ... }`, typed blocks `Key = Type { ... }` (the type is the block's name, as the
// reference's getNodeName returns it), and values `Key = token token ...` up to the end of the
// line.  Keys compare case-insensitively, '#' starts a comment, and single- or double-quoted
// strings are one token.  Errors (unbalanced braces, missing values, wrong value types) throw
// fnet::Error with the line number.
#pragma once

#include <string>
#include <vector>

namespace fnet {
namespace hsd {

struct Node {
  std::string name;                // the key as written
  std::string type;                // typed block: `Key = Type {...}`
  std::vector<std::string> tokens;  // value tokens (quotes removed)
  std::vector<Node> children;       // block contents, in input order
  bool block = false;
  int line = 0;

  // first child named `key` (case-insensitive), or nullptr
  const Node *find(const std::string &key) const;
  // every child named `key`, in input order
  std::vector<const Node *> all(const std::string &key) const;
  // the child's content for a path "A/B/C" (nullptr if absent)
  const Node *path(const std::string &p) const;

  // typed accessors of a value child (with a default when the child is absent)
  std::string str(const std::string &key, const std::string &dflt) const;
  std::string str(const std::string &key) const;  // required
  double real(const std::string &key, double dflt) const;
  double real(const std::string &key) const;
  long long integer(const std::string &key, long long dflt) const;
  long long integer(const std::string &key) const;
  bool logical(const std::string &key, bool dflt) const;
  std::vector<long long> integers(const std::string &key) const;  // required, one or more
};

Node parse(const std::string &text);
Node parseFile(const std::string &path);
std::string lower(std::string s);

}  // namespace hsd
}  // namespace fnet
