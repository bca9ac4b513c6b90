// OpenFOAM case files on the host: the polyMesh (points, faces, owner,
// neighbour, boundary) and the boundaryField of the D field, read from the
// ASCII format OpenFOAM writes, and a polyMesh writer.
//
// The reader stands in for OpenFOAM's polyMesh constructor (the five files
// of constant/polyMesh) and for primitiveMesh's geometry, so that a caller
// without OpenFOAM can hand a meshed case to s4g_mesh_upload.  Of the D
// file it reads the two patch types the solve path builds:
//   fixedDisplacement  value                       (fixedDisplacementFvPatchVectorField.C:156-186)
//   solidTraction      traction, pressure,         (solidTractionFvPatchVectorField.C:58-209)
//                      relaxationFactor
// and rejects everything else by name.  A polyMesh with `empty` patches is
// read as a 2-D mesh without their faces (s4g_foam_empty_direction).
//
// Format handled: a FoamFile header dictionary (format ascii), C and C++
// comments, dictionaries `key value;` and `key { ... }`, lists `N ( ... )`,
// `( ... )` and `N{v}`, `uniform v`, `nonuniform List<T> N ( ... )`, faces
// as `faceList` (`n(a b c)`) or `faceCompactList` (offsets, then labels).

#include "s4g.h"
#include "host_geometry.hpp"
#include "s4g_internal.hpp"

#include <algorithm>
#include <cerrno>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <regex>
#include <sstream>
#include <string>
#include <vector>

struct s4g_foam_case {
  // mesh
  int nPoints = 0, nCells = 0, nFaces = 0, nInt = 0;
  std::vector<double> points;              // [nPoints][3]
  std::vector<int> faceStart, facePoints;  // CSR of the faces' points
  std::vector<int> owner, neighbour;
  std::vector<double> C, V, Cf, Sf;
  std::vector<std::string> patchName, patchType;
  std::vector<std::vector<std::string>> patchGroups;  // inGroups
  std::vector<int> patchStart, patchSize;
  // 2-D: the empty patches' faces are taken out of the mesh above (as they
  // have no faces in OpenFOAM's discretisation); their names stay for the
  // writers, and emptyDir (1, 2, 3: x, y, z; 0: 3-D) is their normal
  std::vector<std::string> emptyPatches;
  int emptyDir = 0;
  // A load series: an interpolationTable, (time value) pairs with
  // increasing times, linear between them; outside its range by its
  // outOfBounds (clamp, OpenFOAM's default, and warn: the end values; error:
  // refused; repeat: periodic).  Empty t: no series (a constant load).
  struct Series {
    int width = 0;
    int bounds = 0;  // 0 clamp or warn, 1 error, 2 repeat
    std::vector<double> t, v;
    std::string name;
  };
  // D boundary conditions, per patch
  struct Bc {
    bool set = false;
    s4g_bc_type type = S4G_SOLID_TRACTION;
    std::vector<double> vec3, pressure;  // constant values, or a series' end value
    double relax = 1.0;
    Series vecSeries, presSeries;        // traction or displacement; pressure
  };
  std::vector<Bc> bcs;
  // load series read from the D file
  double rampEnd = 0;              // linear ramps from zero: their common end time; 0: none
  bool constantBesideRamp = false; // a constant nonzero load beside them
  int seriesKind = 0;              // 0 none, 1 all linear ramps from zero, 2 other tables
};

namespace {

using namespace s4g_host;

struct FoamError {
  std::string msg;
};

[[noreturn]] void fail(const std::string& msg) { throw FoamError{msg}; }

// A uniform list `N{v}` is expanded item by item, so its size is bounded
// (2^28 items) before anything is stored: a corrupt count must not take
// the host's memory.
constexpr long kMaxUniform = 1L << 28;

// ------------------------------------------------------------- tokens ---

struct Tok {
  enum Kind { Word, Str, Punct } kind;
  std::string s;
  bool is(char c) const { return kind == Punct && s[0] == c; }
};

bool isPunct(char c) {
  return c == '{' || c == '}' || c == '(' || c == ')' || c == '[' || c == ']' || c == ';';
}

std::vector<Tok> tokenize(const std::string& t, const std::string& where) {
  std::vector<Tok> out;
  size_t i = 0, n = t.size();
  while (i < n) {
    char c = t[i];
    if (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\f' || c == '\v') { ++i; continue; }
    if (c == '/' && i + 1 < n && t[i + 1] == '/') {
      while (i < n && t[i] != '\n') ++i;
      continue;
    }
    if (c == '/' && i + 1 < n && t[i + 1] == '*') {
      size_t e = t.find("*/", i + 2);
      if (e == std::string::npos) fail(where + ": unterminated comment");
      i = e + 2;
      continue;
    }
    if (isPunct(c)) { out.push_back({Tok::Punct, std::string(1, c)}); ++i; continue; }
    if (c == '"') {
      std::string s;
      ++i;
      while (i < n && t[i] != '"') {
        if (t[i] == '\\' && i + 1 < n) ++i;
        s += t[i++];
      }
      if (i >= n) fail(where + ": unterminated string");
      ++i;
      out.push_back({Tok::Str, s});
      continue;
    }
    size_t b = i;
    // a word that starts with a letter may hold balanced parentheses, as
    // OpenFOAM's words do (grad(D), div((impK*grad(D))), laplacian(DD,D))
    const bool named = std::isalpha((unsigned char)c) || c == '_';
    for (;;) {
      while (i < n && !isPunct(t[i]) && t[i] != '"' && !(t[i] == ' ' || t[i] == '\t' || t[i] == '\n' ||
                                                            t[i] == '\r' || t[i] == '\f' || t[i] == '\v'))
        ++i;
      if (!(named && i < n && t[i] == '(')) break;
      int depth = 0;
      size_t j = i;
      for (; j < n; ++j) {
        if (t[j] == '(') ++depth;
        else if (t[j] == ')' && --depth == 0) break;
        else if (t[j] == ';' || t[j] == '{' || t[j] == '}' || t[j] == '\n') break;
      }
      if (j >= n || t[j] != ')') break;  // not a balanced group: the word ends here
      i = j + 1;
    }
    out.push_back({Tok::Word, t.substr(b, i - b)});
  }
  return out;
}

std::string readFile(const std::string& path) {
  std::ifstream in(path, std::ios::binary);
  if (!in) fail("cannot open " + path);
  std::stringstream ss;
  ss << in.rdbuf();
  return ss.str();
}

// ------------------------------------------------------- dictionaries ---

struct Entry {
  std::string key;
  bool quoted = false;       // a quoted key is a regular expression
  bool isDict = false;
  std::vector<Tok> val;      // tokens up to the terminating ';'
  std::vector<Entry> sub;    // sub-dictionary
};

struct Cursor {
  const std::vector<Tok>& t;
  size_t p;
  std::string where;
  bool end() const { return p >= t.size(); }
  const Tok& peek() const {
    if (end()) fail(where + ": unexpected end of file");
    return t[p];
  }
  const Tok& next() {
    const Tok& k = peek();
    ++p;
    return k;
  }
  void expect(char c) {
    const Tok& k = next();
    if (!k.is(c)) fail(where + ": expected '" + std::string(1, c) + "', found '" + k.s + "'");
  }
};

std::vector<Entry> parseDict(Cursor& c, bool braced) {
  std::vector<Entry> out;
  for (;;) {
    if (c.end()) {
      if (braced) fail(c.where + ": missing '}'");
      return out;
    }
    if (c.peek().is('}')) {
      if (!braced) fail(c.where + ": unexpected '}'");
      c.next();
      return out;
    }
    const Tok& k = c.next();
    if (k.kind == Tok::Punct) fail(c.where + ": unexpected '" + k.s + "'");
    if (k.kind == Tok::Word && k.s[0] == '#') {
      // a directive (#include "file", #inputMode merge, ...): its argument
      // is skipped; what it would have added is then missing and reported
      if (!c.end() && !c.peek().is(';') && c.peek().kind != Tok::Punct) c.next();
      continue;
    }
    Entry e;
    e.key = k.s;
    e.quoted = k.kind == Tok::Str;
    if (!c.end() && c.peek().is('{')) {
      c.next();
      e.isDict = true;
      e.sub = parseDict(c, true);
    } else {
      int depth = 0;
      for (;;) {
        const Tok& v = c.next();
        if (v.kind == Tok::Punct) {
          char ch = v.s[0];
          if (ch == '(' || ch == '[' || ch == '{') ++depth;
          if (ch == ')' || ch == ']' || ch == '}') {
            if (--depth < 0) fail(c.where + ": unbalanced '" + v.s + "' in entry " + e.key);
          }
          if (ch == ';' && depth == 0) break;
        }
        e.val.push_back(v);
      }
    }
    out.push_back(std::move(e));
  }
}

const Entry* find(const std::vector<Entry>& d, const std::string& key) {
  for (const Entry& e : d)
    if (e.key == key) return &e;
  return nullptr;
}

// The file's tokens after its FoamFile header (format ascii required).
std::vector<Tok> payload(const std::string& path, std::string* cls = nullptr) {
  std::vector<Tok> t = tokenize(readFile(path), path);
  if (t.size() >= 2 && t[0].kind == Tok::Word && t[0].s == "FoamFile" && t[1].is('{')) {
    Cursor c{t, 2, path};
    std::vector<Entry> h = parseDict(c, true);
    if (const Entry* f = find(h, "format"))
      if (!f->val.empty() && f->val[0].s != "ascii")
        fail(path + ": format " + f->val[0].s + " is not read (ASCII only)");
    if (cls)
      if (const Entry* k = find(h, "class"))
        if (!k->val.empty()) *cls = k->val[0].s;
    t.erase(t.begin(), t.begin() + (std::ptrdiff_t)c.p);
  }
  return t;
}

// ------------------------------------------------------------ numbers ---

double toDouble(const Tok& k, const std::string& where) {
  if (k.kind != Tok::Word) fail(where + ": expected a number, found '" + k.s + "'");
  errno = 0;
  char* e = nullptr;
  double v = std::strtod(k.s.c_str(), &e);
  if (e == k.s.c_str() || *e != '\0' || errno == ERANGE) fail(where + ": bad number '" + k.s + "'");
  return v;
}

long toLong(const Tok& k, const std::string& where) {
  if (k.kind != Tok::Word) fail(where + ": expected an integer, found '" + k.s + "'");
  errno = 0;
  char* e = nullptr;
  long v = std::strtol(k.s.c_str(), &e, 10);
  if (e == k.s.c_str() || *e != '\0' || errno == ERANGE) fail(where + ": bad integer '" + k.s + "'");
  return v;
}

int toLabel(const Tok& k, const std::string& where) {
  long v = toLong(k, where);
  if (v < 0 || v > 0x7fffffff) fail(where + ": label out of range: " + k.s);
  return (int)v;
}

bool isInteger(const Tok& k) {
  if (k.kind != Tok::Word || k.s.empty()) return false;
  for (char ch : k.s)
    if (ch < '0' || ch > '9') return false;
  return true;
}

// A list of items: `N ( item ... )`, `( item ... )` or `N{item}`; an
// optional leading `List<...>` word is skipped.  item(c) reads one item.
template <class Item>
void parseList(Cursor& c, Item item) {
  if (!c.end() && c.peek().kind == Tok::Word && c.peek().s.rfind("List<", 0) == 0) c.next();
  long n = -1;
  if (isInteger(c.peek())) n = toLong(c.next(), c.where);
  if (c.peek().is('{')) {
    if (n < 0) fail(c.where + ": a uniform list needs a size");
    if (n > kMaxUniform) fail(c.where + ": uniform list of " + std::to_string(n) + " items is too long");
    c.next();
    size_t at = c.p;
    for (long i = 0; i < n; ++i) {
      c.p = at;
      item(c);
    }
    if (n == 0) {  // skip the item without reading it
      int depth = 0;
      while (!(c.peek().is('}') && depth == 0)) {
        const Tok& k = c.next();
        if (k.is('(')) ++depth;
        if (k.is(')')) --depth;
      }
    }
    c.expect('}');
    return;
  }
  c.expect('(');
  long got = 0;
  while (!c.peek().is(')')) {
    item(c);
    ++got;
  }
  c.next();
  if (n >= 0 && got != n) fail(c.where + ": list of " + std::to_string(n) + " has " + std::to_string(got) + " items");
}

P3 parseVector(Cursor& c) {
  c.expect('(');
  P3 v;
  v.x = toDouble(c.next(), c.where);
  v.y = toDouble(c.next(), c.where);
  v.z = toDouble(c.next(), c.where);
  c.expect(')');
  return v;
}

std::vector<int> parseLabels(Cursor& c) {
  std::vector<int> out;
  parseList(c, [&](Cursor& cc) { out.push_back(toLabel(cc.next(), cc.where)); });
  return out;
}

// ------------------------------------------------- large list files ---
// points, faces, owner and neighbour hold one list each (faceCompactList:
// two), of up to millions of items: they are read straight from the text
// with a pointer scanner, without a token per number.

struct Scan {
  std::string text;
  const char* p;
  const char* e;
  std::string where;
  std::string cls;  // the header's class

  explicit Scan(const std::string& path) : text(readFile(path)), where(path) {
    p = text.data();
    e = p + text.size();
    header();
  }
  void skip() {
    for (;;) {
      while (p < e && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r' || *p == '\f' || *p == '\v')) ++p;
      if (p + 1 < e && p[0] == '/' && p[1] == '/') {
        while (p < e && *p != '\n') ++p;
      } else if (p + 1 < e && p[0] == '/' && p[1] == '*') {
        const char* q = p + 2;
        while (q + 1 < e && !(q[0] == '*' && q[1] == '/')) ++q;
        if (q + 1 >= e) fail(where + ": unterminated comment");
        p = q + 2;
      } else {
        return;
      }
    }
  }
  char peek() {
    skip();
    if (p >= e) fail(where + ": unexpected end of file");
    return *p;
  }
  void expect(char c) {
    if (peek() != c) fail(where + ": expected '" + std::string(1, c) + "', found '" + std::string(1, *p) + "'");
    ++p;
  }
  bool delimiter(const char* q) const {
    return q >= e || *q == ' ' || *q == '\t' || *q == '\n' || *q == '\r' || *q == '\f' ||
           *q == '\v' || isPunct(*q) || *q == '/';
  }
  long integer() {
    skip();
    char* end = nullptr;
    errno = 0;
    long v = std::strtol(p, &end, 10);
    if (end == p || errno == ERANGE || !delimiter(end)) fail(where + ": bad integer near '" + std::string(p, std::min<size_t>(16, (size_t)(e - p))) + "'");
    p = end;
    return v;
  }
  int label() {
    long v = integer();
    if (v < 0 || v > 0x7fffffff) fail(where + ": label out of range: " + std::to_string(v));
    return (int)v;
  }
  double number() {
    skip();
    char* end = nullptr;
    errno = 0;
    double v = std::strtod(p, &end);
    if (end == p || errno == ERANGE || !delimiter(end)) fail(where + ": bad number near '" + std::string(p, std::min<size_t>(16, (size_t)(e - p))) + "'");
    p = end;
    return v;
  }
  // The FoamFile header dictionary, if any: format ascii required; class kept.
  void header() {
    skip();
    static const char kw[] = "FoamFile";
    if ((size_t)(e - p) < sizeof(kw) - 1 || std::strncmp(p, kw, sizeof(kw) - 1) != 0) return;
    const char* b = p;
    p += sizeof(kw) - 1;
    expect('{');
    int depth = 1;
    while (depth > 0) {
      skip();
      if (p >= e) fail(where + ": unterminated FoamFile header");
      if (*p == '"') {
        ++p;
        while (p < e && *p != '"') ++p;
      }
      if (p < e && *p == '{') ++depth;
      if (p < e && *p == '}') --depth;
      ++p;
    }
    std::vector<Tok> t = tokenize(std::string(b, p), where);
    Cursor c{t, 2, where};
    std::vector<Entry> h = parseDict(c, true);
    if (const Entry* f = find(h, "format"))
      if (!f->val.empty() && f->val[0].s != "ascii")
        fail(where + ": format " + f->val[0].s + " is not read (ASCII only)");
    if (const Entry* k = find(h, "class"))
      if (!k->val.empty()) cls = k->val[0].s;
  }
};

// `N ( item ... )`, `( item ... )` or `N{item}`, with an optional leading
// List<...> word; item(s) reads one item.
template <class Item>
void scanList(Scan& s, Item item) {
  if (s.peek() == 'L') {
    while (!s.delimiter(s.p)) ++s.p;
  }
  long n = -1;
  if (s.peek() >= '0' && s.peek() <= '9') n = s.integer();
  if (s.peek() == '{') {
    if (n < 0) fail(s.where + ": a uniform list needs a size");
    if (n > kMaxUniform) fail(s.where + ": uniform list of " + std::to_string(n) + " items is too long");
    ++s.p;
    const char* at = s.p;
    for (long i = 0; i < n; ++i) {
      s.p = at;
      item(s);
    }
    if (n == 0)  // an empty list: its one item is not read
      while (s.peek() != '}') ++s.p;
    s.expect('}');
    return;
  }
  s.expect('(');
  long got = 0;
  while (s.peek() != ')') {
    item(s);
    ++got;
  }
  ++s.p;
  if (n >= 0 && got != n)
    fail(s.where + ": list of " + std::to_string(n) + " has " + std::to_string(got) + " items");
}

std::vector<int> scanLabels(Scan& s) {
  std::vector<int> out;
  scanList(s, [&](Scan& ss) { out.push_back(ss.label()); });
  return out;
}

// ----------------------------------------------------------- polyMesh ---

// 2-D meshes: the faces of `empty` patches leave the mesh (the cell centres
// and volumes are already those of the closed cells).  The empty patches
// must be normal to x, y or z, and every cell must have two such faces
// (one cell across the empty direction), as OpenFOAM requires.
void takeOutEmptyPatches(s4g_foam_case& m, const std::string& where) {
  std::vector<char> isEmpty(m.patchName.size(), 0);
  bool any = false;
  for (size_t p = 0; p < m.patchName.size(); ++p)
    if (m.patchType[p] == "empty") isEmpty[p] = 1, any = true;
  if (!any) return;
  int dir = 0;
  std::vector<int> perCell((size_t)m.nCells, 0);
  for (size_t p = 0; p < m.patchName.size(); ++p) {
    if (!isEmpty[p]) continue;
    for (int i = 0; i < m.patchSize[p]; ++i) {
      const int f = m.patchStart[p] + i;
      const double* S = &m.Sf[3 * (size_t)f];
      const double mS = std::sqrt(S[0] * S[0] + S[1] * S[1] + S[2] * S[2]);
      int k = -1;
      for (int a = 0; a < 3; ++a)
        if (mS > 0 && std::fabs(std::fabs(S[a]) / mS - 1.0) < 1e-6) k = a + 1;
      if (k < 0 || (dir && k != dir))
        fail(where + ": empty patch " + m.patchName[p] + " is not normal to x, y or z");
      dir = k;
      perCell[(size_t)m.owner[(size_t)f]]++;
    }
  }
  for (int c = 0; c < m.nCells; ++c)
    if (perCell[(size_t)c] != 2)
      fail(where + ": a 2-D mesh needs one cell across the empty direction (two empty faces per cell)");
  // compact the faces, keeping the order of the others
  std::vector<int> owner, faceStart{0}, facePoints, pStart, pSize;
  std::vector<double> Cf, Sf;
  std::vector<std::string> names, types;
  std::vector<std::vector<std::string>> groups;
  auto keep = [&](int f) {
    owner.push_back(m.owner[(size_t)f]);
    for (int k = 0; k < 3; ++k) {
      Cf.push_back(m.Cf[3 * (size_t)f + k]);
      Sf.push_back(m.Sf[3 * (size_t)f + k]);
    }
    facePoints.insert(facePoints.end(), m.facePoints.begin() + m.faceStart[(size_t)f],
                      m.facePoints.begin() + m.faceStart[(size_t)f + 1]);
    faceStart.push_back((int)facePoints.size());
  };
  for (int f = 0; f < m.nInt; ++f) keep(f);
  for (size_t p = 0; p < m.patchName.size(); ++p) {
    if (isEmpty[p]) {
      m.emptyPatches.push_back(m.patchName[p]);
      continue;
    }
    pStart.push_back((int)owner.size());
    pSize.push_back(m.patchSize[p]);
    names.push_back(m.patchName[p]);
    types.push_back(m.patchType[p]);
    groups.push_back(m.patchGroups[p]);
    for (int i = 0; i < m.patchSize[p]; ++i) keep(m.patchStart[p] + i);
  }
  m.owner.swap(owner); m.Cf.swap(Cf); m.Sf.swap(Sf);
  m.faceStart.swap(faceStart); m.facePoints.swap(facePoints);
  m.patchStart.swap(pStart); m.patchSize.swap(pSize);
  m.patchName.swap(names); m.patchType.swap(types); m.patchGroups.swap(groups);
  m.nFaces = (int)m.owner.size();
  m.bcs.assign(m.patchName.size(), s4g_foam_case::Bc{});
  m.emptyDir = dir;
}

void readMesh(s4g_foam_case& m, const std::string& dir) {
  {  // points
    Scan s(dir + "/points");
    scanList(s, [&](Scan& ss) {
      ss.expect('(');
      for (int k = 0; k < 3; ++k) m.points.push_back(ss.number());
      ss.expect(')');
    });
    m.nPoints = (int)(m.points.size() / 3);
  }
  {  // faces
    Scan s(dir + "/faces");
    m.faceStart.assign(1, 0);
    if (s.cls == "faceCompactList") {
      std::vector<int> offsets = scanLabels(s);
      m.facePoints = scanLabels(s);
      if (offsets.empty() || offsets[0] != 0 || offsets.back() != (int)m.facePoints.size())
        fail(s.where + ": faceCompactList offsets do not match its labels");
      for (size_t f = 1; f < offsets.size(); ++f) {
        if (offsets[f] < offsets[f - 1]) fail(s.where + ": decreasing faceCompactList offsets");
        m.faceStart.push_back(offsets[f]);
      }
    } else {
      scanList(s, [&](Scan& ss) {
        scanList(ss, [&](Scan& s3) { m.facePoints.push_back(s3.label()); });
        m.faceStart.push_back((int)m.facePoints.size());
      });
    }
    m.nFaces = (int)m.faceStart.size() - 1;
  }
  {
    Scan s(dir + "/owner");
    m.owner = scanLabels(s);
  }
  {
    Scan s(dir + "/neighbour");
    m.neighbour = scanLabels(s);
  }
  {  // boundary: N ( name { type ..; nFaces ..; startFace ..; } ... )
    std::string path = dir + "/boundary";
    std::vector<Tok> t = payload(path);
    Cursor c{t, 0, path};
    if (isInteger(c.peek())) c.next();
    c.expect('(');
    while (!c.peek().is(')')) {
      const Tok& name = c.next();
      if (name.kind == Tok::Punct) fail(path + ": expected a patch name");
      c.expect('{');
      std::vector<Entry> d = parseDict(c, true);
      const Entry* ty = find(d, "type");
      const Entry* nf = find(d, "nFaces");
      const Entry* sf = find(d, "startFace");
      if (!ty || !nf || !sf || ty->val.empty() || nf->val.size() != 1 || sf->val.size() != 1)
        fail(path + ": patch " + name.s + " needs type, nFaces and startFace");
      m.patchName.push_back(name.s);
      m.patchType.push_back(ty->val[0].s);
      std::vector<std::string> groups;
      if (const Entry* g = find(d, "inGroups"))
        for (const Tok& k : g->val)
          if (k.kind == Tok::Word && !isInteger(k) && k.s.rfind("List<", 0) != 0) groups.push_back(k.s);
      m.patchGroups.push_back(groups);
      m.patchSize.push_back(toLabel(nf->val[0], path));
      m.patchStart.push_back(toLabel(sf->val[0], path));
    }
    c.next();
  }

  // consistency
  const std::string where = dir;
  m.nInt = (int)m.neighbour.size();
  if ((int)m.owner.size() != m.nFaces)
    fail(where + ": owner has " + std::to_string(m.owner.size()) + " labels for " + std::to_string(m.nFaces) + " faces");
  if (m.nInt > m.nFaces) fail(where + ": more neighbours than faces");
  int maxCell = -1;
  for (int v : m.owner) maxCell = std::max(maxCell, v);
  for (int v : m.neighbour) maxCell = std::max(maxCell, v);
  m.nCells = maxCell + 1;
  if (m.nCells < 1) fail(where + ": no cells");
  for (int p : m.facePoints)
    if (p >= m.nPoints) fail(where + ": face point label " + std::to_string(p) + " out of range");
  for (int f = 0; f < m.nFaces; ++f)
    if (m.faceStart[f + 1] - m.faceStart[f] < 3) fail(where + ": face " + std::to_string(f) + " has fewer than 3 points");
  int expect = m.nInt;
  for (size_t p = 0; p < m.patchName.size(); ++p) {
    if (m.patchStart[p] != expect)
      fail(where + ": patch " + m.patchName[p] + " does not start where the previous one ends");
    expect += m.patchSize[p];
  }
  if (expect != m.nFaces) fail(where + ": the patches do not cover the boundary faces");

  // geometry
  m.Cf.assign(3 * (size_t)m.nFaces, 0.0);
  m.Sf.assign(3 * (size_t)m.nFaces, 0.0);
  std::vector<P3> poly;
  for (int f = 0; f < m.nFaces; ++f) {
    const int b = m.faceStart[f], n = m.faceStart[f + 1] - b;
    poly.resize((size_t)n);
    for (int i = 0; i < n; ++i) {
      const double* q = &m.points[3 * (size_t)m.facePoints[b + i]];
      poly[(size_t)i] = P3{q[0], q[1], q[2]};
    }
    P3 ctr, area;
    if (n == 3) {  // primitiveMesh takes triangles directly
      ctr = scl(1.0 / 3.0, add(add(poly[0], poly[1]), poly[2]));
      area = scl(0.5, cross(sub(poly[1], poly[0]), sub(poly[2], poly[0])));
    } else {
      polygonGeometry(poly.data(), n, ctr, area);
    }
    m.Cf[3 * (size_t)f] = ctr.x; m.Cf[3 * (size_t)f + 1] = ctr.y; m.Cf[3 * (size_t)f + 2] = ctr.z;
    m.Sf[3 * (size_t)f] = area.x; m.Sf[3 * (size_t)f + 1] = area.y; m.Sf[3 * (size_t)f + 2] = area.z;
  }
  m.C.assign(3 * (size_t)m.nCells, 0.0);
  m.V.assign((size_t)m.nCells, 0.0);
  if (!cellGeometry(m.nCells, m.nFaces, m.nInt, m.owner.data(), m.neighbour.data(), m.Cf.data(),
                    m.Sf.data(), m.C.data(), m.V.data()))
    fail(where + ": a cell has no faces or a volume that is not positive");
  takeOutEmptyPatches(m, where);
  m.bcs.assign(m.patchName.size(), s4g_foam_case::Bc{});
}

// ----------------------------------------------------------------- D ---

// `uniform v` or `nonuniform List<T> N (...)` of width 1 or 3, for n faces.
std::vector<double> fieldValues(const Entry& e, int width, int n, const std::string& where) {
  std::vector<double> out;
  Cursor c{e.val, 0, where + " " + e.key};
  if (c.end()) fail(c.where + ": empty entry");
  const Tok& form = c.next();
  auto item = [&](Cursor& cc) {
    if (width == 3) {
      P3 v = parseVector(cc);
      out.push_back(v.x); out.push_back(v.y); out.push_back(v.z);
    } else {
      out.push_back(toDouble(cc.next(), cc.where));
    }
  };
  if (form.s == "uniform") {
    item(c);
    std::vector<double> one = out;
    out.clear();
    for (int i = 0; i < n; ++i) out.insert(out.end(), one.begin(), one.end());
  } else if (form.s == "nonuniform") {
    parseList(c, item);
    if ((int)out.size() != width * n)
      fail(c.where + ": " + std::to_string(out.size() / width) + " values for " + std::to_string(n) + " faces");
  } else {
    fail(c.where + ": expected uniform or nonuniform, found '" + form.s + "'");
  }
  if (!c.end()) fail(c.where + ": unexpected '" + c.peek().s + "'");
  return out;
}

// The patch's entry, in OpenFOAM's order: its name, then one of its groups
// (inGroups), then a quoted key read as a regular expression ("(left|right)",
// ".*"), the last such key first.
const Entry* patchEntry(const std::vector<Entry>& bf, const std::string& name,
                        const std::vector<std::string>& groups) {
  if (const Entry* e = find(bf, name)) return e;
  for (const std::string& g : groups)
    if (const Entry* e = find(bf, g)) return e;
  for (auto it = bf.rbegin(); it != bf.rend(); ++it) {
    if (!it->quoted) continue;
    try {
      if (std::regex_match(name, std::regex(it->key))) return &*it;
    } catch (const std::regex_error&) {
    }
  }
  return nullptr;
}

// A dictionary entry by name, else by a quoted key whose regular expression
// matches the name (OpenFOAM's "fileName|file").
const Entry* lookup(const std::vector<Entry>& d, const std::string& name) {
  if (const Entry* e = find(d, name)) return e;
  for (auto it = d.rbegin(); it != d.rend(); ++it) {
    if (!it->quoted) continue;
    try {
      if (std::regex_match(name, std::regex(it->key))) return &*it;
    } catch (const std::regex_error&) {
    }
  }
  return nullptr;
}

std::string expandCase(std::string s, const std::string& caseDir) {
  for (const char* var : {"${FOAM_CASE}", "$FOAM_CASE"}) {
    size_t at;
    while ((at = s.find(var)) != std::string::npos) s.replace(at, std::strlen(var), caseDir);
  }
  return s;
}

struct Ramp {
  double end = 0;
  std::vector<double> value;  // the value at the end, width 1 or 3
};

// A load series (interpolationTable) read from its file; ramp says whether
// it is a linear ramp from zero at time 0 -- what the load increments apply
// (load factor n/N) -- with its end time and end value.
s4g_foam_case::Series readSeries(const Entry& series, int width, const std::string& caseDir,
                                 const std::string& where, bool* ramp, Ramp* r) {
  if (!series.isDict) fail(where + ": " + series.key + " must be a dictionary");
  const Entry* f = lookup(series.sub, "file");
  if (!f) f = lookup(series.sub, "fileName");
  if (!f || f->val.size() != 1) fail(where + ": " + series.key + " has no file");
  if (const Entry* is = lookup(series.sub, "interpolationScheme"))
    if (!is->val.empty() && is->val[0].s != "linear")
      fail(where + ": " + series.key + ": interpolationScheme " + is->val[0].s + " is not built");
  s4g_foam_case::Series out;
  out.width = width;
  out.name = where + ": " + series.key;
  if (const Entry* ob = lookup(series.sub, "outOfBounds")) {
    const std::string b = ob->val.empty() ? std::string() : ob->val[0].s;
    if (b == "clamp" || b == "warn") out.bounds = 0;
    else if (b == "error") out.bounds = 1;
    else if (b == "repeat") out.bounds = 2;
    else fail(where + ": " + series.key + ": outOfBounds " + b + " is unknown (clamp, warn, error, repeat)");
  }
  const std::string file = expandCase(f->val[0].s, caseDir);
  std::vector<Tok> t = payload(file);
  Cursor c{t, 0, file};
  parseList(c, [&](Cursor& cc) {
    cc.expect('(');
    out.t.push_back(toDouble(cc.next(), cc.where));
    if (width == 3) {
      P3 v = parseVector(cc);
      out.v.push_back(v.x); out.v.push_back(v.y); out.v.push_back(v.z);
    } else {
      out.v.push_back(toDouble(cc.next(), cc.where));
    }
    cc.expect(')');
  });
  const size_t n = out.t.size();
  if (n < 2) fail(file + ": a series needs at least two points");
  for (size_t i = 1; i < n; ++i)
    if (!(out.t[i] > out.t[i - 1])) fail(file + ": times must increase");
  r->end = out.t[n - 1];
  r->value.assign(out.v.end() - width, out.v.end());
  double scale = 0;
  for (double v : r->value) scale = std::max(scale, std::fabs(v));
  *ramp = out.t[0] == 0.0;
  for (size_t i = 0; i < n && *ramp; ++i)
    for (int k = 0; k < width; ++k) {
      const double expect = r->value[(size_t)k] * (out.t[i] / r->end);
      if (std::fabs(out.v[i * width + k] - expect) > 1e-12 * scale + (i == 0 ? 0.0 : 1e-300))
        *ramp = false;
    }
  return out;
}

// The series at time x (linear interpolation between its points).
void seriesAt(const s4g_foam_case::Series& s, double x, double* out) {
  const size_t n = s.t.size();
  const int w = s.width;
  const double t0 = s.t[0], t1 = s.t[n - 1];
  if (s.bounds == 2 && (x < t0 || x > t1)) {
    const double span = t1 - t0;
    x = t0 + std::fmod(x - t0, span);
    if (x < t0) x += span;
  } else if (s.bounds == 1 && (x < t0 || x > t1)) {
    fail(s.name + ": time " + std::to_string(x) + " is outside the series (outOfBounds error)");
  }
  if (x <= t0) {
    for (int k = 0; k < w; ++k) out[k] = s.v[(size_t)k];
    return;
  }
  if (x >= t1) {
    for (int k = 0; k < w; ++k) out[k] = s.v[(n - 1) * w + k];
    return;
  }
  const size_t hi = (size_t)(std::upper_bound(s.t.begin(), s.t.end(), x) - s.t.begin());
  const size_t lo = hi - 1;
  const double f = (x - s.t[lo]) / (s.t[hi] - s.t[lo]);
  for (int k = 0; k < w; ++k) {
    const double a = s.v[lo * w + k], b = s.v[hi * w + k];
    out[k] = a + f * (b - a);
  }
}

void readD(s4g_foam_case& m, const std::string& path) {
  std::vector<Tok> t = payload(path);
  Cursor c{t, 0, path};
  std::vector<Entry> d = parseDict(c, false);
  const Entry* bf = find(d, "boundaryField");
  if (!bf || !bf->isDict) fail(path + ": no boundaryField dictionary");
  // the case directory holds 0/D
  std::string caseDir = path;
  for (int up = 0; up < 2; ++up) {
    size_t at = caseDir.find_last_of('/');
    caseDir = at == std::string::npos ? std::string(".") : caseDir.substr(0, at);
  }
  std::vector<s4g_foam_case::Bc> bcs(m.patchName.size());
  double rampEnd = 0;
  bool anyRamp = false, anyConstantLoad = false, anyTable = false, rampsDiffer = false;
  // a series that is a linear ramp from zero, with the others' end time, is
  // what the load increments apply; any other table is stepped in time
  auto series = [&](const Entry& e, int width, const std::string& where,
                    s4g_foam_case::Series& keep) {
    bool ramp = false;
    Ramp r;
    keep = readSeries(e, width, caseDir, where, &ramp, &r);
    if (ramp) {
      if (anyRamp && r.end != rampEnd) rampsDiffer = true;
      anyRamp = true;
      rampEnd = r.end;
    } else {
      anyTable = true;
    }
    return r;
  };
  auto nonzero = [](const std::vector<double>& v) {
    for (double x : v)
      if (x != 0.0) return true;
    return false;
  };
  auto isOff = [](const Entry* s) {
    return s && !s->val.empty() && (s->val[0].s == "false" || s->val[0].s == "no" || s->val[0].s == "off");
  };
  auto isOn = [](const Entry* s) {
    return s && !s->val.empty() && (s->val[0].s == "true" || s->val[0].s == "yes" || s->val[0].s == "on");
  };
  for (size_t p = 0; p < m.patchName.size(); ++p) {
    const std::string& name = m.patchName[p];
    const std::string where = path + ": patch " + name;
    const Entry* e = patchEntry(bf->sub, name, m.patchGroups[p]);
    if (!e || !e->isDict) fail(where + " has no entry in boundaryField");
    const Entry* ty = find(e->sub, "type");
    if (!ty || ty->val.size() != 1) fail(where + " has no type");
    const std::string type = ty->val[0].s;
    const int n = m.patchSize[p];
    s4g_foam_case::Bc& bc = bcs[p];
    bc.set = true;
    auto tile = [n](const std::vector<double>& v) {
      std::vector<double> out;
      for (int i = 0; i < n; ++i) out.insert(out.end(), v.begin(), v.end());
      return out;
    };
    if (isOff(find(e->sub, "nonOrthogonalCorrections")))
      fail(where + ": nonOrthogonalCorrections false is not built");
    if (type == "fixedDisplacement") {
      bc.type = S4G_FIXED_DISPLACEMENT;
      if (const Entry* ds = find(e->sub, "displacementSeries")) {
        Ramp r = series(*ds, 3, where, bc.vecSeries);
        bc.vec3 = tile(r.value);
      } else {
        const Entry* v = find(e->sub, "value");
        bc.vec3 = v ? fieldValues(*v, 3, n, where) : std::vector<double>(3 * (size_t)n, 0.0);
        anyConstantLoad = anyConstantLoad || nonzero(bc.vec3);
      }
    } else if (type == "solidTraction") {
      bc.type = S4G_SOLID_TRACTION;
      if (isOn(find(e->sub, "setEffectiveTraction"))) fail(where + ": setEffectiveTraction is not built");
      // exactly one of each (solidTractionFvPatchVectorField.C:105-193)
      for (const char* q : {"traction", "pressure"}) {
        const std::string k(q);
        const Entry* plain = find(e->sub, k);
        const Entry* ser = find(e->sub, k + "Series");
        const Entry* field = find(e->sub, k + "Field");
        if ((plain != nullptr) + (ser != nullptr) + (field != nullptr) > 1)
          fail(where + ": only one of " + k + ", " + k + "Series or " + k + "Field can be specified");
        if (field) fail(where + ": " + k + "Field is not built");
        std::vector<double>& out = k == "traction" ? bc.vec3 : bc.pressure;
        const int width = k == "traction" ? 3 : 1;
        if (ser) {
          Ramp r = series(*ser, width, where, k == "traction" ? bc.vecSeries : bc.presSeries);
          out = tile(r.value);
        } else {
          if (!plain) fail(where + ": solidTraction needs " + k);
          out = fieldValues(*plain, width, n, where);
          anyConstantLoad = anyConstantLoad || nonzero(out);
        }
      }
      if (const Entry* rf = find(e->sub, "relaxationFactor")) {
        if (rf->val.size() != 1) fail(where + ": bad relaxationFactor");
        bc.relax = toDouble(rf->val[0], where);
        if (!(bc.relax > 0.0 && bc.relax <= 1.0)) fail(where + ": relaxationFactor must be in (0, 1]");
      }
    } else {
      fail(where + ": type " + type + " is not built (fixedDisplacement and solidTraction are)");
    }
  }
  m.bcs = std::move(bcs);
  // ramps that end at different times are stepped in time like tables
  m.seriesKind = (anyTable || rampsDiffer) ? 2 : anyRamp ? 1 : 0;
  m.rampEnd = m.seriesKind == 1 ? rampEnd : 0.0;
  m.constantBesideRamp = m.seriesKind == 1 && anyConstantLoad;
}

// ------------------------------------------------------------- writer ---

bool writeFile(const std::string& path, const std::string& cls, const std::string& object,
               const std::string& body) {
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  std::fprintf(f,
               "FoamFile\n{\n    version     2.0;\n    format      ascii;\n"
               "    class       %s;\n    location    \"constant/polyMesh\";\n"
               "    object      %s;\n}\n\n",
               cls.c_str(), object.c_str());
  std::fwrite(body.data(), 1, body.size(), f);
  bool ok = std::fclose(f) == 0;
  return ok;
}

std::string labels(const int* v, int n) {
  std::string s = std::to_string(n) + "\n(\n";
  for (int i = 0; i < n; ++i) s += std::to_string(v[i]) + "\n";
  return s + ")\n";
}

s4g_status guarded(const std::function<void()>& body) {
  try {
    body();
    return S4G_OK;
  } catch (const FoamError& e) {
    s4g::setLastError(e.msg);
    return S4G_BAD_ARG;
  } catch (const std::bad_alloc&) {
    s4g::setLastError("out of host memory reading an OpenFOAM case");
    return S4G_OOM;
  }
}

}  // namespace

extern "C" {

s4g_status s4g_foam_read_mesh(const char* polymesh_dir, s4g_foam_case** out) {
  if (!polymesh_dir || !out) return S4G_BAD_ARG;
  *out = nullptr;
  auto* m = new s4g_foam_case();
  s4g_status st = guarded([&] { readMesh(*m, polymesh_dir); });
  if (st != S4G_OK) {
    delete m;
    return st;
  }
  *out = m;
  return S4G_OK;
}

s4g_status s4g_foam_mesh_desc(const s4g_foam_case* m, s4g_mesh_desc* d, int* n_points) {
  if (!m || !d) return S4G_BAD_ARG;
  d->n_cells = m->nCells;
  d->n_faces = m->nFaces;
  d->n_internal_faces = m->nInt;
  d->owner = m->owner.data();
  d->neighbour = m->neighbour.data();
  d->C = m->C.data();
  d->V = m->V.data();
  d->Cf = m->Cf.data();
  d->Sf = m->Sf.data();
  d->n_patches = (int)m->patchName.size();
  d->patch_start = m->patchStart.data();
  d->patch_size = m->patchSize.data();
  if (n_points) *n_points = m->nPoints;
  return S4G_OK;
}

s4g_status s4g_foam_mesh_points(const s4g_foam_case* m, const double** points,
                                const int** face_start, const int** face_points) {
  if (!m) return S4G_BAD_ARG;
  if (points) *points = m->points.data();
  if (face_start) *face_start = m->faceStart.data();
  if (face_points) *face_points = m->facePoints.data();
  return S4G_OK;
}

const char* s4g_foam_patch_name(const s4g_foam_case* m, int p) {
  if (!m || p < 0 || p >= (int)m->patchName.size()) return nullptr;
  return m->patchName[(size_t)p].c_str();
}

const char* s4g_foam_patch_type(const s4g_foam_case* m, int p) {
  if (!m || p < 0 || p >= (int)m->patchType.size()) return nullptr;
  return m->patchType[(size_t)p].c_str();
}

s4g_status s4g_foam_read_d(s4g_foam_case* m, const char* d_file) {
  if (!m || !d_file) return S4G_BAD_ARG;
  return guarded([&] { readD(*m, d_file); });
}

s4g_status s4g_foam_bc(const s4g_foam_case* m, int p, s4g_bc_type* type, const double** vec3,
                       const double** pressure, double* relaxation_factor) {
  if (!m || p < 0 || p >= (int)m->bcs.size()) return S4G_BAD_ARG;
  const s4g_foam_case::Bc& bc = m->bcs[(size_t)p];
  if (!bc.set) {
    s4g::setLastError("no D file has been read for this case");
    return S4G_BAD_ARG;
  }
  if (type) *type = bc.type;
  if (vec3) *vec3 = bc.vec3.data();
  if (pressure) *pressure = bc.type == S4G_SOLID_TRACTION ? bc.pressure.data() : nullptr;
  if (relaxation_factor) *relaxation_factor = bc.relax;
  return S4G_OK;
}

s4g_status s4g_foam_apply_bcs(const s4g_foam_case* m, s4g_mesh* mesh) {
  if (!m || !mesh) return S4G_BAD_ARG;
  for (size_t p = 0; p < m->bcs.size(); ++p) {
    const s4g_foam_case::Bc& bc = m->bcs[p];
    if (!bc.set) {
      s4g::setLastError("no D file has been read for this case");
      return S4G_BAD_ARG;
    }
    s4g_status st = s4g_bc_set(mesh, (int)p, bc.type, bc.vec3.data(),
                               bc.type == S4G_SOLID_TRACTION ? bc.pressure.data() : nullptr);
    if (st != S4G_OK) return st;
    if (bc.type == S4G_SOLID_TRACTION) {
      st = s4g_bc_set_relaxation(mesh, (int)p, bc.relax);
      if (st != S4G_OK) return st;
    }
  }
  return S4G_OK;
}

s4g_status s4g_foam_read_time(const char* control_dict, double* start_time, double* end_time,
                              double* delta_t) {
  if (!control_dict) return S4G_BAD_ARG;
  return guarded([&] {
    std::vector<Tok> t = payload(control_dict);
    Cursor c{t, 0, control_dict};
    std::vector<Entry> d = parseDict(c, false);
    auto num = [&](const char* key, double dflt, bool required) {
      const Entry* e = find(d, key);
      if (!e) {
        if (required) fail(std::string(control_dict) + ": no " + key);
        return dflt;
      }
      if (e->val.size() != 1) fail(std::string(control_dict) + ": bad " + key);
      return toDouble(e->val[0], control_dict);
    };
    const double t0 = num("startTime", 0.0, false), t1 = num("endTime", 0.0, true),
                 dt = num("deltaT", 0.0, true);
    if (!(dt > 0) || !(t1 > t0)) fail(std::string(control_dict) + ": need endTime > startTime and deltaT > 0");
    if (start_time) *start_time = t0;
    if (end_time) *end_time = t1;
    if (delta_t) *delta_t = dt;
  });
}

s4g_status s4g_foam_read_relaxation(const char* fv_solution, const char* field,
                                    double* field_factor, double* equation_factor) {
  if (!fv_solution || !field) return S4G_BAD_ARG;
  return guarded([&] {
    std::vector<Tok> t = payload(fv_solution);
    Cursor c{t, 0, fv_solution};
    std::vector<Entry> d = parseDict(c, false);
    double ff = 1.0, ef = 1.0;
    auto factor = [&](const Entry* e) {
      if (!e || e->isDict || e->val.size() != 1) fail(std::string(fv_solution) + ": bad relaxation factor");
      return toDouble(e->val[0], fv_solution);
    };
    if (const Entry* rf = find(d, "relaxationFactors")) {
      if (!rf->isDict) fail(std::string(fv_solution) + ": relaxationFactors must be a dictionary");
      const Entry* fields = find(rf->sub, "fields");
      const Entry* eqns = find(rf->sub, "equations");
      if (fields || eqns) {
        if (fields && fields->isDict)
          if (const Entry* e = lookup(fields->sub, field)) ff = factor(e);
        if (eqns && eqns->isDict)
          if (const Entry* e = lookup(eqns->sub, field)) ef = factor(e);
      } else if (const Entry* e = lookup(rf->sub, field)) {
        ff = factor(e);  // the older form: field factors directly in relaxationFactors
      }
    }
    if (field_factor) *field_factor = ff;
    if (equation_factor) *equation_factor = ef;
  });
}

s4g_status s4g_foam_read_grad_scheme(const char* fv_schemes, const char* field,
                                     int* ls_boundary_delta) {
  if (!fv_schemes || !field || !ls_boundary_delta) return S4G_BAD_ARG;
  return guarded([&] {
    std::vector<Tok> t = payload(fv_schemes);
    Cursor c{t, 0, fv_schemes};
    std::vector<Entry> d = parseDict(c, false);
    const std::string w = std::string(fv_schemes) + ": gradSchemes";
    const Entry* gs = find(d, "gradSchemes");
    if (!gs || !gs->isDict) fail(w + " missing");
    const std::string key = std::string("grad(") + field + ")";
    const Entry* e = lookup(gs->sub, key);
    if (!e || (e->val.size() == 1 && e->val[0].s == "none")) e = find(gs->sub, "default");
    if (!e || e->isDict || e->val.empty() || e->val[0].s == "none") fail(w + ": no scheme for " + key);
    const std::string name = e->val[0].s;
    // leastSquares: OpenFOAM's patch delta, normal to the patch;
    // extendedLeastSquares: the full face-centre delta on the boundary
    // (with minDet the scheme's threshold for adding neighbours, which the
    // hexahedral and prismatic meshes here never reach)
    if (name == "leastSquares" && e->val.size() == 1) *ls_boundary_delta = 0;
    else if (name == "extendedLeastSquares" && e->val.size() == 2) *ls_boundary_delta = 1;
    else fail(w + ": " + key + " " + name + " is not built (leastSquares and extendedLeastSquares are)");
  });
}

s4g_status s4g_foam_read_controls(const char* case_dir, s4g_model* model, s4g_law* law,
                                  s4g_lin_solver* lin, s4g_outer* outer) {
  if (!case_dir || !model || !law || !lin || !outer) return S4G_BAD_ARG;
  return guarded([&] {
    const std::string dir(case_dir);
    auto readDict = [](const std::string& path) {
      std::vector<Tok> t = payload(path);
      Cursor c{t, 0, path};
      return parseDict(c, false);
    };
    // a number: the last token of `key value;`, `key [dims] value;` or
    // `key name [dims] value;` (a dimensionedScalar)
    auto number = [](const Entry* e, const std::string& where) {
      if (!e || e->isDict || e->val.empty()) fail(where + ": missing or bad entry");
      return toDouble(e->val.back(), where + " " + e->key);
    };
    // constant/solidProperties: solidModel and <model>Coeffs (solidModel.C:909-912)
    const std::string sp = dir + "/constant/solidProperties";
    std::vector<Entry> props = readDict(sp);
    const Entry* sm = find(props, "solidModel");
    if (!sm || sm->val.size() != 1) fail(sp + ": no solidModel");
    const std::string name = sm->val[0].s;
    if (name == "linearGeometryTotalDisplacement") *model = S4G_LIN_GEOM_TOTAL_DISP;
    else if (name == "nonLinearGeometryTotalLagrangian") *model = S4G_NONLIN_GEOM_TOTAL_LAG;
    else if (name == "nonLinearGeometryTotalLagrangianTotalDisplacement")
      *model = S4G_NONLIN_GEOM_TOTAL_LAG_TOTAL_DISP;
    else fail(sp + ": solidModel " + name + " is not built");
    s4g_default_controls(lin, outer);
    if (const Entry* co = lookup(props, name + "Coeffs")) {
      if (!co->isDict) fail(sp + ": " + name + "Coeffs must be a dictionary");
      const std::string w = sp + ": " + name + "Coeffs";
      if (const Entry* e = find(co->sub, "nCorrectors")) outer->n_correctors = (int)number(e, w);
      if (const Entry* e = find(co->sub, "solutionTolerance")) outer->solution_tol = number(e, w);
      if (const Entry* e = find(co->sub, "alternativeTolerance")) outer->alternative_tol = number(e, w);
      if (const Entry* e = find(co->sub, "materialTolerance")) outer->material_tol = number(e, w);
      if (const Entry* e = find(co->sub, "infoFrequency")) outer->info_frequency = (int)number(e, w);
      if (const Entry* st = find(co->sub, "stabilisation")) {
        if (!st->isDict) fail(w + ": stabilisation must be a dictionary");
        const Entry* ty = find(st->sub, "type");
        if (ty && (ty->val.size() != 1 || ty->val[0].s != "RhieChow"))
          fail(w + ": stabilisation type " + (ty->val.empty() ? "" : ty->val[0].s) + " is not built");
        if (const Entry* e = find(st->sub, "scaleFactor")) outer->stab_scale = number(e, w);
      }
      if (const Entry* e = find(co->sub, "relaxationMethod")) {
        const std::string m = e->val.size() == 1 ? e->val[0].s : "";
        if (m == "fixed") outer->relaxation_method = 0;
        else if (m == "Aitken") outer->relaxation_method = 1;
        else fail(w + ": relaxationMethod " + m + " is unknown (fixed or Aitken)");
      }
      for (const char* k : {"predictor", "solvePressureEqn"})
        if (const Entry* e = find(co->sub, k))
          if (!e->val.empty() && (e->val[0].s == "yes" || e->val[0].s == "true" || e->val[0].s == "on"))
            fail(w + ": " + k + " is not built");
    }
    // constant/mechanicalProperties: one law (linearElastic.C:62-89,
    // neoHookeanElastic.C:50-79); planeStress must be no
    const std::string mp = dir + "/constant/mechanicalProperties";
    std::vector<Entry> mech = readDict(mp);
    const Entry* ps = find(mech, "planeStress");
    if (ps && !ps->val.empty() && (ps->val[0].s == "yes" || ps->val[0].s == "true" || ps->val[0].s == "on"))
      fail(mp + ": planeStress yes is not built");
    const Entry* laws = find(mech, "mechanical");
    if (!laws || laws->isDict) fail(mp + ": no mechanical ( ... ) list");
    // the list holds `name { ... }` sub-dictionaries: parse its tokens
    std::vector<Tok> lt(laws->val.begin(), laws->val.end());
    if (lt.size() < 2 || !lt.front().is('(') || !lt.back().is(')')) fail(mp + ": bad mechanical list");
    std::vector<Tok> inner(lt.begin() + 1, lt.end() - 1);
    Cursor lc{inner, 0, mp};
    std::vector<Entry> list = parseDict(lc, false);
    if (list.size() != 1 || !list[0].isDict)
      fail(mp + ": " + std::to_string(list.size()) + " laws; one law is built");
    const std::vector<Entry>& ld = list[0].sub;
    const Entry* ty = find(ld, "type");
    if (!ty || ty->val.size() != 1) fail(mp + ": the law has no type");
    *law = s4g_law{};
    if (ty->val[0].s == "linearElastic") law->type = S4G_LINEAR_ELASTIC;
    else if (ty->val[0].s == "neoHookeanElastic") law->type = S4G_NEO_HOOKEAN;
    else fail(mp + ": law type " + ty->val[0].s + " is not built");
    const Entry *E = find(ld, "E"), *nu = find(ld, "nu"), *mu = find(ld, "mu"), *K = find(ld, "K");
    if (E && nu && !(law->type == S4G_NEO_HOOKEAN && (mu || K))) {
      law->E = number(E, mp);
      law->nu = number(nu, mp);
    } else if (mu && K && !(law->type == S4G_NEO_HOOKEAN && (E || nu))) {
      law->use_mu_K = 1;
      law->mu = number(mu, mp);
      law->K = number(K, mp);
    } else {
      fail(mp + ": give E and nu, or mu and K");
    }
    if (const Entry* rho = find(ld, "rho")) law->rho = number(rho, mp);
    if (find(ld, "sigma0")) fail(mp + ": sigma0 is not built");
    // system/fvSolution: the solved field's solver (lduMatrix::solver::New)
    const std::string fs = dir + "/system/fvSolution";
    std::vector<Entry> sol = readDict(fs);
    const char* field = *model == S4G_NONLIN_GEOM_TOTAL_LAG ? "DD" : "D";
    const Entry* solvers = find(sol, "solvers");
    const Entry* sd = solvers && solvers->isDict ? lookup(solvers->sub, field) : nullptr;
    if (!sd || !sd->isDict) fail(fs + ": no solver for " + field);
    const std::string w = fs + ": solver for " + field;
    const Entry* sv = find(sd->sub, "solver");
    if (!sv || sv->val.size() != 1 || sv->val[0].s != "PCG")
      fail(w + ": solver " + (sv && !sv->val.empty() ? sv->val[0].s : std::string("?")) +
           " is not built (PCG is)");
    const Entry* pc = find(sd->sub, "preconditioner");
    const std::string pname = pc && !pc->isDict && pc->val.size() == 1 ? pc->val[0].s : "";
    if (pname == "DIC" || pname == "FDIC") lin->preconditioner = S4G_PRECOND_DIC;
    else if (pname == "diagonal") lin->preconditioner = S4G_PRECOND_DIAGONAL;
    else fail(w + ": preconditioner " + pname + " is not built (DIC, FDIC and diagonal are)");
    if (const Entry* e = find(sd->sub, "tolerance")) lin->tolerance = number(e, w);
    if (const Entry* e = find(sd->sub, "relTol")) lin->rel_tol = number(e, w);
    if (const Entry* e = find(sd->sub, "maxIter")) lin->max_iter = (int)number(e, w);
    // relaxationFactors { fields { D f; } } (solidModel.C:837-841 via D.relax());
    // an equation factor is returned by s4g_foam_read_relaxation for the caller
    double ff = 1.0, ef = 1.0;
    if (s4g_foam_read_relaxation(fs.c_str(), field, &ff, &ef) != S4G_OK)
      fail(fs + ": bad relaxationFactors");
    if (!(ff > 0.0 && ff <= 1.0)) fail(fs + ": field relaxation factor must be in (0, 1]");
    outer->field_relaxation = ff;
  });
}

s4g_status s4g_foam_load_ramp(const s4g_foam_case* m, double* end_time, int* constant_loads) {
  if (!m) return S4G_BAD_ARG;
  if (end_time) *end_time = m->rampEnd;
  if (constant_loads) *constant_loads = m->constantBesideRamp ? 1 : 0;
  return S4G_OK;
}

s4g_status s4g_foam_series_kind(const s4g_foam_case* m, int* kind) {
  if (!m || !kind) return S4G_BAD_ARG;
  *kind = m->seriesKind;
  return S4G_OK;
}

s4g_status s4g_foam_bc_at(const s4g_foam_case* m, int p, double time, s4g_bc_type* type,
                          double* vec3, double* pressure, double* relaxation_factor) {
  if (!m || p < 0 || p >= (int)m->bcs.size()) return S4G_BAD_ARG;
  const s4g_foam_case::Bc& bc = m->bcs[(size_t)p];
  if (!bc.set) {
    s4g::setLastError("no D file has been read for this case");
    return S4G_BAD_ARG;
  }
  return guarded([&] {
    const size_t n = (size_t)m->patchSize[(size_t)p];
    if (type) *type = bc.type;
    if (relaxation_factor) *relaxation_factor = bc.relax;
    if (vec3) {
      if (bc.vecSeries.t.empty()) {
        std::copy(bc.vec3.begin(), bc.vec3.end(), vec3);
      } else {
        double v[3];
        seriesAt(bc.vecSeries, time, v);
        for (size_t i = 0; i < n; ++i)
          for (int k = 0; k < 3; ++k) vec3[3 * i + k] = v[k];
      }
    }
    if (pressure && bc.type == S4G_SOLID_TRACTION) {
      if (bc.presSeries.t.empty()) {
        std::copy(bc.pressure.begin(), bc.pressure.end(), pressure);
      } else {
        double v;
        seriesAt(bc.presSeries, time, &v);
        for (size_t i = 0; i < n; ++i) pressure[i] = v;
      }
    }
  });
}

s4g_status s4g_foam_apply_bcs_at(const s4g_foam_case* m, s4g_mesh* mesh, double time) {
  if (!m || !mesh) return S4G_BAD_ARG;
  std::vector<double> v, pr;
  for (size_t p = 0; p < m->bcs.size(); ++p) {
    const size_t n = (size_t)m->patchSize[p];
    v.assign(3 * n, 0.0);
    pr.assign(n, 0.0);
    s4g_bc_type type;
    double rf = 1.0;
    s4g_status st = s4g_foam_bc_at(m, (int)p, time, &type, v.data(), pr.data(), &rf);
    if (st != S4G_OK) return st;
    st = s4g_bc_set(mesh, (int)p, type, v.data(), type == S4G_SOLID_TRACTION ? pr.data() : nullptr);
    if (st != S4G_OK) return st;
    if (type == S4G_SOLID_TRACTION) {
      st = s4g_bc_set_relaxation(mesh, (int)p, rf);
      if (st != S4G_OK) return st;
    }
  }
  return S4G_OK;
}

void s4g_foam_free(s4g_foam_case* m) { delete m; }

s4g_status s4g_foam_boundary_D(const s4g_foam_case* m, const double* D, const double* gradD,
                               double* Db) {
  if (!m || !D || !gradD || !Db) return S4G_BAD_ARG;
  for (size_t p = 0; p < m->patchName.size(); ++p) {
    const s4g_foam_case::Bc* bc = p < m->bcs.size() && m->bcs[p].set ? &m->bcs[p] : nullptr;
    for (int i = 0; i < m->patchSize[p]; ++i) {
      const int f = m->patchStart[p] + i, b = f - m->nInt, c = m->owner[(size_t)f];
      double* out = Db + 3 * (size_t)b;
      if (bc && bc->type == S4G_FIXED_DISPLACEMENT) {
        for (int k = 0; k < 3; ++k) out[k] = bc->vec3[3 * (size_t)i + k];
        continue;
      }
      // D_P + (C_f - C_P) . gradD_P, gradD_ij = dD_j/dx_i
      const double* g = gradD + 9 * (size_t)c;
      double d[3];
      for (int k = 0; k < 3; ++k) d[k] = m->Cf[3 * (size_t)f + k] - m->C[3 * (size_t)c + k];
      for (int j = 0; j < 3; ++j)
        out[j] = D[3 * (size_t)c + j] + d[0] * g[j] + d[1] * g[3 + j] + d[2] * g[6 + j];
    }
  }
  return S4G_OK;
}

s4g_status s4g_foam_write_field(const s4g_foam_case* m, const char* dir, const char* name, int width,
                                const char* dimensions, const double* cell_values,
                                const double* boundary_values) {
  if (!m || !dir || !name || !cell_values || (width != 1 && width != 3 && width != 6))
    return S4G_BAD_ARG;
  const char* cls = width == 1 ? "volScalarField" : width == 3 ? "volVectorField" : "volSymmTensorField";
  const char* list = width == 1 ? "scalar" : width == 3 ? "vector" : "symmTensor";
  std::string d(dir);
  while (d.size() > 1 && d.back() == '/') d.pop_back();
  const std::string time = d.substr(d.find_last_of('/') + 1);
  const std::string path = d + "/" + name;
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) {
    s4g::setLastError("cannot write " + path);
    return S4G_BAD_ARG;
  }
  auto value = [&](const double* v) {
    if (width == 1) {
      std::fprintf(f, "%.12g\n", v[0]);
    } else {
      std::fputc('(', f);
      for (int k = 0; k < width; ++k) std::fprintf(f, k ? " %.12g" : "%.12g", v[k]);
      std::fputs(")\n", f);
    }
  };
  std::fprintf(f,
               "FoamFile\n{\n    version     2.0;\n    format      ascii;\n    class       %s;\n"
               "    location    \"%s\";\n    object      %s;\n}\n"
               "// Boundary values: %s.\n\n"
               "dimensions      %s;\n\ninternalField   nonuniform List<%s>\n%d\n(\n",
               cls, time.c_str(), name,
               boundary_values ? "supplied with the field (for D from s4g_foam_boundary_D: the "
                                 "prescribed value on fixedDisplacement patches, elsewhere the "
                                 "cell value extrapolated with its gradient)"
                               : "those of the adjacent cells",
               dimensions ? dimensions : "[0 0 0 0 0 0 0]", list, m->nCells);
  for (int c = 0; c < m->nCells; ++c) value(cell_values + (size_t)width * c);
  std::fputs(")\n;\n\nboundaryField\n{\n", f);
  for (size_t p = 0; p < m->patchName.size(); ++p) {
    std::fprintf(f, "    %s\n    {\n", m->patchName[p].c_str());
    if (m->patchType[p] == "empty") {
      std::fputs("        type            empty;\n    }\n", f);
      continue;
    }
    std::fprintf(f, "        type            calculated;\n        value           nonuniform List<%s>\n%d\n(\n",
                 list, m->patchSize[p]);
    for (int i = 0; i < m->patchSize[p]; ++i) {
      const int face = m->patchStart[p] + i;
      value(boundary_values ? boundary_values + (size_t)width * (face - m->nInt)
                            : cell_values + (size_t)width * m->owner[(size_t)face]);
    }
    std::fputs(")\n;\n    }\n", f);
  }
  for (const std::string& e : m->emptyPatches)
    std::fprintf(f, "    %s\n    {\n        type            empty;\n    }\n", e.c_str());
  std::fputs("}\n", f);
  if (std::fclose(f) != 0) {
    s4g::setLastError("cannot write " + path);
    return S4G_BAD_ARG;
  }
  return S4G_OK;
}

int s4g_foam_empty_direction(const s4g_foam_case* m) { return m ? m->emptyDir : 0; }

s4g_status s4g_foam_write_point_field(const s4g_foam_case* m, const char* dir, const char* name,
                                      const char* dimensions, const double* values) {
  if (!m || !dir || !name || !values) return S4G_BAD_ARG;
  std::string d(dir);
  while (d.size() > 1 && d.back() == '/') d.pop_back();
  const std::string time = d.substr(d.find_last_of('/') + 1);
  const std::string path = d + "/" + name;
  FILE* f = std::fopen(path.c_str(), "w");
  if (!f) {
    s4g::setLastError("cannot write " + path);
    return S4G_BAD_ARG;
  }
  std::fprintf(f,
               "FoamFile\n{\n    version     2.0;\n    format      ascii;\n"
               "    class       pointVectorField;\n    location    \"%s\";\n    object      %s;\n}\n\n"
               "dimensions      %s;\n\ninternalField   nonuniform List<vector>\n%d\n(\n",
               time.c_str(), name, dimensions ? dimensions : "[0 1 0 0 0 0 0]", m->nPoints);
  for (int i = 0; i < m->nPoints; ++i)
    std::fprintf(f, "(%.12g %.12g %.12g)\n", values[3 * (size_t)i], values[3 * (size_t)i + 1],
                 values[3 * (size_t)i + 2]);
  std::fputs(")\n;\n\nboundaryField\n{\n", f);
  for (const std::string& p : m->patchName)
    std::fprintf(f, "    %s\n    {\n        type            calculated;\n    }\n", p.c_str());
  for (const std::string& e : m->emptyPatches)
    std::fprintf(f, "    %s\n    {\n        type            empty;\n    }\n", e.c_str());
  std::fputs("}\n", f);
  if (std::fclose(f) != 0) {
    s4g::setLastError("cannot write " + path);
    return S4G_BAD_ARG;
  }
  return S4G_OK;
}

s4g_status s4g_foam_write_mesh(const char* dir, int n_points, const double* points, int n_faces,
                               const int* face_start, const int* face_points, int n_int,
                               const int* owner, const int* neighbour, int n_patches,
                               const char* const* names, const int* patch_start,
                               const int* patch_size, const char* const* types) {
  if (!dir || n_points < 0 || n_faces < 0 || n_int < 0 || n_int > n_faces || n_patches < 0 ||
      !points || !face_start || !face_points || !owner || (n_int > 0 && !neighbour) ||
      (n_patches > 0 && (!names || !patch_start || !patch_size)))
    return S4G_BAD_ARG;
  const std::string d(dir);
  char buf[128];
  std::string s = std::to_string(n_points) + "\n(\n";
  for (int i = 0; i < n_points; ++i) {
    std::snprintf(buf, sizeof buf, "(%.17g %.17g %.17g)\n", points[3 * (size_t)i],
                  points[3 * (size_t)i + 1], points[3 * (size_t)i + 2]);
    s += buf;
  }
  s += ")\n";
  if (!writeFile(d + "/points", "vectorField", "points", s)) return S4G_BAD_ARG;
  s = std::to_string(n_faces) + "\n(\n";
  for (int f = 0; f < n_faces; ++f) {
    s += std::to_string(face_start[f + 1] - face_start[f]) + "(";
    for (int k = face_start[f]; k < face_start[f + 1]; ++k)
      s += std::to_string(face_points[k]) + (k + 1 < face_start[f + 1] ? " " : "");
    s += ")\n";
  }
  s += ")\n";
  if (!writeFile(d + "/faces", "faceList", "faces", s)) return S4G_BAD_ARG;
  if (!writeFile(d + "/owner", "labelList", "owner", labels(owner, n_faces))) return S4G_BAD_ARG;
  if (!writeFile(d + "/neighbour", "labelList", "neighbour", labels(neighbour, n_int)))
    return S4G_BAD_ARG;
  s = std::to_string(n_patches) + "\n(\n";
  for (int p = 0; p < n_patches; ++p)
    s += std::string("    ") + names[p] + "\n    {\n        type            " +
         (types && types[p] ? types[p] : "patch") + ";\n        nFaces          " +
         std::to_string(patch_size[p]) + ";\n        startFace       " + std::to_string(patch_start[p]) +
         ";\n    }\n";
  s += ")\n";
  if (!writeFile(d + "/boundary", "polyBoundaryMesh", "boundary", s)) return S4G_BAD_ARG;
  return S4G_OK;
}

}  // extern "C"
