// HSD input subset of the fnet program (see hsd.hpp).
#include "hsd.hpp"

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <sstream>

#include "fnet_host.hpp"

namespace fnet {
namespace hsd {

namespace {

struct Tok {
  std::string text;
  bool quoted = false;
  bool newline_before = false;  // a line break separates it from the previous token
  int line = 0;
};

std::vector<Tok> tokenize(const std::string &s) {
  std::vector<Tok> out;
  int line = 1;
  bool nl = true;
  size_t i = 0;
  while (i < s.size()) {
    const char c = s[i];
    if (c == '\n') {
      line++;
      nl = true;
      i++;
    } else if (std::isspace((unsigned char)c)) {
      i++;
    } else if (c == '#') {
      while (i < s.size() && s[i] != '\n') i++;
    } else if (c == '{' || c == '}' || c == '=') {
      out.push_back(Tok{std::string(1, c), false, nl, line});
      nl = false;
      i++;
    } else if (c == '\'' || c == '"') {
      const size_t j = s.find(c, i + 1);
      if (j == std::string::npos) throw Error(FNETG_E_INVALID, "HSD: unterminated string at line " + std::to_string(line));
      out.push_back(Tok{s.substr(i + 1, j - i - 1), true, nl, line});
      for (size_t k = i; k < j; k++) line += s[k] == '\n';
      nl = false;
      i = j + 1;
    } else {
      size_t j = i;
      while (j < s.size() && !std::isspace((unsigned char)s[j]) && s[j] != '{' && s[j] != '}' &&
             s[j] != '=' && s[j] != '#')
        j++;
      out.push_back(Tok{s.substr(i, j - i), false, nl, line});
      nl = false;
      i = j;
    }
  }
  return out;
}

[[noreturn]] void fail(const std::string &msg, int line) {
  throw Error(FNETG_E_INVALID, "HSD: " + msg + (line ? " (line " + std::to_string(line) + ")" : ""));
}

bool is_punct(const Tok &t) { return !t.quoted && (t.text == "{" || t.text == "}" || t.text == "="); }

// block contents up to the matching '}' (or the end of input for the top level)
void parse_block(const std::vector<Tok> &t, size_t &i, Node &parent, bool top) {
  while (i < t.size()) {
    if (!t[i].quoted && t[i].text == "}") {
      if (top) fail("unbalanced '}'", t[i].line);
      i++;
      return;
    }
    if (is_punct(t[i])) fail("unexpected '" + t[i].text + "'", t[i].line);
    Node n;
    n.name = t[i].text;
    n.line = t[i].line;
    i++;
    if (i < t.size() && !t[i].quoted && t[i].text == "{") {
      i++;
      n.block = true;
      parse_block(t, i, n, false);
    } else if (i < t.size() && !t[i].quoted && t[i].text == "=") {
      i++;
      if (i >= t.size()) fail("missing value of '" + n.name + "'", n.line);
      if (i + 1 < t.size() && !t[i + 1].quoted && t[i + 1].text == "{" && !t[i].quoted) {
        n.type = t[i].text;
        n.block = true;
        i += 2;
        parse_block(t, i, n, false);
      } else {
        // value tokens up to the end of the line
        n.tokens.push_back(t[i].text);
        i++;
        while (i < t.size() && !t[i].newline_before && !is_punct(t[i])) {
          n.tokens.push_back(t[i].text);
          i++;
        }
      }
    } else {
      fail("'" + n.name + "' is neither a block nor a value", n.line);
    }
    parent.children.push_back(std::move(n));
  }
  if (!top) fail("missing '}'", 0);
}

const Node &required(const Node &n, const std::string &key) {
  const Node *c = n.find(key);
  if (!c) fail("missing '" + key + "' in '" + n.name + "'", n.line);
  return *c;
}

std::string joined(const Node &c) {
  if (c.block || c.tokens.empty()) fail("'" + c.name + "' needs a value", c.line);
  std::string s;
  for (size_t k = 0; k < c.tokens.size(); k++) s += (k ? " " : "") + c.tokens[k];
  return s;
}

double to_real(const Node &c) {
  const std::string s = joined(c);
  char *end = nullptr;
  std::string t = s;
  for (char &ch : t)
    if (ch == 'd' || ch == 'D') ch = 'e';  // Fortran exponent letter
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str() || *end) fail("'" + c.name + "' is not a real number: " + s, c.line);
  return v;
}

long long to_int(const Node &c, const std::string &s) {
  char *end = nullptr;
  const long long v = std::strtoll(s.c_str(), &end, 10);
  if (end == s.c_str() || *end) fail("'" + c.name + "' is not an integer: " + s, c.line);
  return v;
}

}  // namespace

std::string lower(std::string s) {
  for (char &c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

const Node *Node::find(const std::string &key) const {
  const std::string k = lower(key);
  for (const Node &c : children)
    if (lower(c.name) == k) return &c;
  return nullptr;
}

std::vector<const Node *> Node::all(const std::string &key) const {
  std::vector<const Node *> out;
  const std::string k = lower(key);
  for (const Node &c : children)
    if (lower(c.name) == k) out.push_back(&c);
  return out;
}

const Node *Node::path(const std::string &p) const {
  const Node *n = this;
  std::stringstream ss(p);
  std::string part;
  while (n && std::getline(ss, part, '/'))
    if (!part.empty()) n = n->find(part);
  return n;
}

std::string Node::str(const std::string &key, const std::string &dflt) const {
  const Node *c = find(key);
  return c ? joined(*c) : dflt;
}
std::string Node::str(const std::string &key) const { return joined(required(*this, key)); }

double Node::real(const std::string &key, double dflt) const {
  const Node *c = find(key);
  return c ? to_real(*c) : dflt;
}
double Node::real(const std::string &key) const { return to_real(required(*this, key)); }

long long Node::integer(const std::string &key, long long dflt) const {
  const Node *c = find(key);
  return c ? to_int(*c, joined(*c)) : dflt;
}
long long Node::integer(const std::string &key) const {
  const Node &c = required(*this, key);
  return to_int(c, joined(c));
}

bool Node::logical(const std::string &key, bool dflt) const {
  const Node *c = find(key);
  if (!c) return dflt;
  const std::string v = lower(joined(*c));
  if (v == "yes" || v == "true" || v == ".true.") return true;
  if (v == "no" || v == "false" || v == ".false.") return false;
  fail("'" + c->name + "' must be Yes or No", c->line);
}

std::vector<long long> Node::integers(const std::string &key) const {
  const Node &c = required(*this, key);
  if (c.block || c.tokens.empty()) fail("'" + key + "' needs values", c.line);
  std::vector<long long> out;
  for (const std::string &s : c.tokens) out.push_back(to_int(c, s));
  return out;
}

Node parse(const std::string &text) {
  const std::vector<Tok> t = tokenize(text);
  Node root;
  root.name = "(input)";
  root.block = true;
  size_t i = 0;
  parse_block(t, i, root, true);
  return root;
}

Node parseFile(const std::string &path) {
  std::ifstream in(path);
  if (!in) throw Error(FNETG_E_INVALID, "cannot open " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  return parse(ss.str());
}

}  // namespace hsd
}  // namespace fnet
