// scene.cpp -- scene files in the reference's XML vocabulary, and TetGen volume meshes.
//
// The reference reads FEM volumes, the problem type, solver options and boundary conditions
// from XML with per-component loaders (source/PhySim/Utils/Serializer_XML.cpp):
//   LoadSimulable_VolumeFEM  :1199-1325   meshInit / meshRest, discretization, shapeFunction,
//                                          materialParam, materialModel, quadrature
//   LoadDistribution         :618-733     CONSTANT / VARIABLE distributions over elements
//   LoadDistributed          :376-616     the parameter sets, material models, shape
//                                          functions and quadratures they hold
//   LoadMesh_TetVolume       :878-983     FILEVOLUME meshes with position / scale / rotation
//   LoadOptimProblem         :1327-1354   Static, or Dynamic with its step
//   LoadOptimSolver          :1356-1505   iteration limits, step type, linear solver, line search
//   LoadBoundary             :1507-1647   Gravity and FixPosition (hard or soft, numStep,
//                                          Transform3D animation, geometry selections :1758-1868)
// It ships no top-level reader that calls them, so this file defines the one document layout
// that holds them: a root element with the children <simulable> (the LoadSimulable_VolumeFEM
// element), <problem>, <solver> and <boundary> (its <bc> children), each read with the
// reference's own element and attribute names, defaults and quirks (noted where they apply).
// Everything the tet-FEM Newton path does not solve (other discretizations, shape functions,
// material models, contact planes, surface meshes that need TetGen's mesher) is refused
// with a message rather than approximated.
//
// The reference declares a TetGen volume reader (Serializer_Mesh::ReadVolume_TET,
// include/PhySim/Utils/Serializer_Mesh.h:46-52) without defining it; FILEVOLUME meshes are
// read here from TetGen's published .node / .ele formats.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/phx.h"
#include "errors.h"

namespace {

// ---------------------------------------------------------------------------
// a small XML reader: elements, attributes, character data, comments, CDATA and the five
// predefined entities (plus numeric character references); no DTD processing
// ---------------------------------------------------------------------------
struct XNode {
  std::string name;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::vector<std::unique_ptr<XNode>> kids;
  std::string text;
  const std::string* attr(const char* a) const {
    for (auto& kv : attrs)
      if (kv.first == a) return &kv.second;
    return nullptr;
  }
  const XNode* child(const char* c) const {
    for (auto& k : kids)
      if (k->name == c) return k.get();
    return nullptr;
  }
  std::vector<const XNode*> children(const char* c) const {
    std::vector<const XNode*> out;
    for (auto& k : kids)
      if (k->name == c) out.push_back(k.get());
    return out;
  }
};

struct XParser {
  const std::string& s;
  size_t i = 0;
  std::string err;
  explicit XParser(const std::string& src) : s(src) {}

  bool fail(const std::string& m) {
    if (err.empty()) {
      size_t line = 1 + std::count(s.begin(), s.begin() + std::min(i, s.size()), '\n');
      err = "XML line " + std::to_string(line) + ": " + m;
    }
    return false;
  }
  bool starts(const char* t) const { return s.compare(i, std::strlen(t), t) == 0; }
  void ws() {
    while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
  }
  bool skip_to(const char* t) {
    size_t p = s.find(t, i);
    if (p == std::string::npos) return fail(std::string("unterminated construct, expected ") + t);
    i = p + std::strlen(t);
    return true;
  }
  // comments, processing instructions and declarations between elements
  bool misc() {
    for (;;) {
      ws();
      if (starts("<!--")) {
        if (!skip_to("-->")) return false;
      } else if (starts("<?")) {
        if (!skip_to("?>")) return false;
      } else if (starts("<!DOCTYPE")) {
        if (!skip_to(">")) return false;
      } else {
        return true;
      }
    }
  }
  static bool name_char(char c) { return std::isalnum((unsigned char)c) || c == '_' || c == '-' || c == '.' || c == ':'; }
  bool name(std::string& out) {
    size_t b = i;
    while (i < s.size() && name_char(s[i])) ++i;
    if (i == b) return fail("expected a name");
    out = s.substr(b, i - b);
    return true;
  }
  bool decode(const std::string& raw, std::string& out) {
    out.clear();
    for (size_t k = 0; k < raw.size(); ++k) {
      if (raw[k] != '&') {
        out += raw[k];
        continue;
      }
      size_t e = raw.find(';', k);
      if (e == std::string::npos) return fail("unterminated entity");
      std::string ent = raw.substr(k + 1, e - k - 1);
      if (ent == "lt") out += '<';
      else if (ent == "gt") out += '>';
      else if (ent == "amp") out += '&';
      else if (ent == "quot") out += '"';
      else if (ent == "apos") out += '\'';
      else if (!ent.empty() && ent[0] == '#') {
        long v = ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X') ? std::strtol(ent.c_str() + 2, nullptr, 16)
                                                                    : std::strtol(ent.c_str() + 1, nullptr, 10);
        if (v <= 0 || v > 127) return fail("character reference outside ASCII: &" + ent + ";");
        out += (char)v;
      } else {
        return fail("unknown entity &" + ent + ";");
      }
      k = e;
    }
    return true;
  }
  bool element(XNode& n, int depth) {
    if (depth > 64) return fail("elements nested too deeply");
    if (!starts("<")) return fail("expected an element");
    ++i;
    if (!name(n.name)) return false;
    for (;;) {
      ws();
      if (starts("/>")) {
        i += 2;
        return true;
      }
      if (starts(">")) {
        ++i;
        break;
      }
      std::string an, av;
      if (!name(an)) return false;
      ws();
      if (!starts("=")) return fail("expected '=' after attribute " + an);
      ++i;
      ws();
      if (i >= s.size() || (s[i] != '"' && s[i] != '\'')) return fail("expected a quoted value for " + an);
      const char q = s[i++];
      size_t e = s.find(q, i);
      if (e == std::string::npos) return fail("unterminated attribute value");
      if (!decode(s.substr(i, e - i), av)) return false;
      i = e + 1;
      n.attrs.emplace_back(an, av);
    }
    // content
    for (;;) {
      if (i >= s.size()) return fail("element <" + n.name + "> is not closed");
      if (starts("</")) {
        i += 2;
        std::string cn;
        if (!name(cn)) return false;
        if (cn != n.name) return fail("</" + cn + "> closes <" + n.name + ">");
        ws();
        if (!starts(">")) return fail("expected '>'");
        ++i;
        return true;
      }
      if (starts("<!--")) {
        if (!skip_to("-->")) return false;
        continue;
      }
      if (starts("<![CDATA[")) {
        i += 9;
        size_t e = s.find("]]>", i);
        if (e == std::string::npos) return fail("unterminated CDATA");
        n.text += s.substr(i, e - i);
        i = e + 3;
        continue;
      }
      if (starts("<?")) {
        if (!skip_to("?>")) return false;
        continue;
      }
      if (starts("<")) {
        n.kids.emplace_back(new XNode());
        if (!element(*n.kids.back(), depth + 1)) return false;
        continue;
      }
      size_t e = s.find('<', i);
      if (e == std::string::npos) e = s.size();
      std::string t;
      if (!decode(s.substr(i, e - i), t)) return false;
      n.text += t;
      i = e;
    }
  }
  bool document(XNode& root) {
    if (s.size() >= 3 && (unsigned char)s[0] == 0xEF && (unsigned char)s[1] == 0xBB && (unsigned char)s[2] == 0xBF) i = 3;
    if (!misc()) return false;
    if (!element(root, 0)) return false;
    if (!misc()) return false;
    if (i != s.size()) return fail("content after the root element");
    return true;
  }
};

bool read_file(const std::string& path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

// IOUtils::stringToVector_CSV: numbers separated by commas (whitespace and line breaks allowed)
bool csv_numbers(const std::string& t, std::vector<double>& out) {
  out.clear();
  std::string tok;
  auto flush = [&]() -> bool {
    if (tok.empty()) return true;
    char* end = nullptr;
    const double v = std::strtod(tok.c_str(), &end);
    if (!end || *end != '\0') return false;
    out.push_back(v);
    tok.clear();
    return true;
  };
  for (char c : t) {
    if (c == ',' || c == ';' || std::isspace((unsigned char)c)) {
      if (!flush()) return false;
    } else {
      tok += c;
    }
  }
  return flush();
}

std::string dir_of(const std::string& p) {
  size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string(".") : p.substr(0, k);
}
std::string resolve(const std::string& p, const std::string& dir) {
  if (!p.empty() && p[0] == '/') return p;
  return dir + "/" + p;
}

// ---------------------------------------------------------------------------
// TetGen .node / .ele
// ---------------------------------------------------------------------------
// Lines of a TetGen file without comments ('#' to the end of a line) and blank lines.
bool tetgen_lines(const std::string& path, std::vector<std::vector<double>>& rows, std::string& err) {
  std::string src;
  if (!read_file(path, src)) {
    err = "cannot read " + path;
    return false;
  }
  std::istringstream in(src);
  std::string line;
  while (std::getline(in, line)) {
    const size_t h = line.find('#');
    if (h != std::string::npos) line.resize(h);
    std::istringstream ls(line);
    std::vector<double> r;
    std::string tok;
    while (ls >> tok) {
      char* end = nullptr;
      const double v = std::strtod(tok.c_str(), &end);
      if (!end || *end != '\0') {
        err = path + ": not a number: " + tok;
        return false;
      }
      r.push_back(v);
    }
    if (!r.empty()) rows.push_back(std::move(r));
  }
  if (rows.empty()) {
    err = path + ": empty";
    return false;
  }
  return true;
}

// Reads <base>.node and <base>.ele (TetGen's formats: a header line with the counts, then one
// line per point "index x y z [attributes] [marker]" and per tetrahedron "index n0 n1 n2 n3
// [region]"; indices start at 0 or 1, as the first point's index says).  Tetrahedra with a
// negative signed volume are reoriented (corners 1 and 2 swapped): the path needs positive
// rest volumes, as the reference's inverted-element guard does (EnergyElement_FEM.cpp:126-131).
bool read_tetgen(const std::string& path, std::vector<double>& V, std::vector<int32_t>& T, int* flipped,
                 std::string& err) {
  std::string base = path;
  for (const char* ext : {".node", ".ele", ".face"}) {
    const size_t L = std::strlen(ext);
    if (base.size() > L && base.compare(base.size() - L, L, ext) == 0) {
      base.resize(base.size() - L);
      break;
    }
  }
  std::vector<std::vector<double>> nr, er;
  if (!tetgen_lines(base + ".node", nr, err) || !tetgen_lines(base + ".ele", er, err)) return false;
  const auto& nh = nr[0];
  if (nh.size() < 2 || nh[1] != 3) {
    err = base + ".node: the header must give the point count and dimension 3";
    return false;
  }
  const long np = (long)nh[0];
  const int nattr = nh.size() > 2 ? (int)nh[2] : 0;
  if (np <= 0 || (long)nr.size() - 1 < np) {
    err = base + ".node: fewer points than the header announces";
    return false;
  }
  const long first = (long)nr[1][0];
  if (first != 0 && first != 1) {
    err = base + ".node: point indices must start at 0 or 1";
    return false;
  }
  V.assign(3 * (size_t)np, 0.0);
  for (long k = 0; k < np; ++k) {
    const auto& r = nr[1 + k];
    if ((long)r[0] != first + k || (int)r.size() < 4 + nattr) {
      err = base + ".node: point line " + std::to_string(k) + " is malformed";
      return false;
    }
    for (int c = 0; c < 3; ++c) V[3 * k + c] = r[1 + c];
  }
  const auto& eh = er[0];
  if (eh.size() < 2) {
    err = base + ".ele: the header must give the tetrahedron count and nodes per tetrahedron";
    return false;
  }
  const long ne = (long)eh[0];
  const int per = (int)eh[1];
  if (per != 4) {
    err = base + ".ele: " + std::to_string(per) + "-node tetrahedra (only the 4-node Tet4 element is solved)";
    return false;
  }
  if (ne <= 0 || (long)er.size() - 1 < ne) {
    err = base + ".ele: fewer tetrahedra than the header announces";
    return false;
  }
  T.assign(4 * (size_t)ne, 0);
  int flips = 0;
  for (long e = 0; e < ne; ++e) {
    const auto& r = er[1 + e];
    if ((int)r.size() < 5) {
      err = base + ".ele: tetrahedron line " + std::to_string(e) + " is malformed";
      return false;
    }
    for (int a = 0; a < 4; ++a) {
      const long id = (long)r[1 + a] - first;
      if (id < 0 || id >= np) {
        err = base + ".ele: node index out of range in tetrahedron " + std::to_string(e);
        return false;
      }
      T[4 * e + a] = (int32_t)id;
    }
    const double* x0 = &V[3 * (size_t)T[4 * e]];
    double D[9];
    for (int c = 0; c < 3; ++c)
      for (int r2 = 0; r2 < 3; ++r2) D[r2 + 3 * c] = V[3 * (size_t)T[4 * e + 1 + c] + r2] - x0[r2];
    const double det = D[0] * (D[4] * D[8] - D[7] * D[5]) - D[3] * (D[1] * D[8] - D[7] * D[2]) +
                       D[6] * (D[1] * D[5] - D[4] * D[2]);
    if (det < 0) {
      std::swap(T[4 * e + 1], T[4 * e + 2]);
      ++flips;
    }
  }
  if (flipped) *flipped = flips;
  return true;
}

// ---------------------------------------------------------------------------
// the scene
// ---------------------------------------------------------------------------
struct Mat3 {
  double a[9];  // row-major
};
Mat3 mul(const Mat3& A, const Mat3& B) {
  Mat3 C{};
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < 3; ++k) C.a[3 * r + c] += A.a[3 * r + k] * B.a[3 * k + c];
  return C;
}
// GeometryUtils::rotationEulerToMatrix (GeometryUtils.cpp:79-114): R = Rz Ry Rx, radians
Mat3 euler(const double v[3]) {
  const double cx = std::cos(v[0]), sx = std::sin(v[0]), cy = std::cos(v[1]), sy = std::sin(v[1]);
  const double cz = std::cos(v[2]), sz = std::sin(v[2]);
  const Mat3 Rx{{1, 0, 0, 0, cx, -sx, 0, sx, cx}}, Ry{{cy, 0, sy, 0, 1, 0, -sy, 0, cy}}, Rz{{cz, -sz, 0, sz, cz, 0, 0, 0, 1}};
  return mul(Rz, mul(Ry, Rx));
}

}  // namespace

struct phx_scene_s {
  int32_t n = 0, m = 0;
  std::vector<double> X0, x_init, lame, rho, soft_k, soft_t;
  std::vector<int32_t> T;
  std::vector<uint8_t> model, fixed;
  double gravity[3] = {0, 0, 0};
  phx_options opts{};
  int32_t dynamic = 0;
  double dt = 0.0;
  int32_t num_stages = 0;
  struct Group {
    phx_stage_group g;
    std::vector<int32_t> nodes;
  };
  std::vector<Group> groups;
  int32_t flipped = 0;
};

namespace {

struct Loader {
  std::string dir, err;
  bool fail(const std::string& m) {
    if (err.empty()) err = m;
    return false;
  }
  bool vec3(const XNode* n, double out[3], const char* what) {
    std::vector<double> v;
    if (!n || !csv_numbers(n->text, v) || v.size() != 3)
      return fail(std::string("expected a CSV 3D vector in <") + what + ">");
    for (int c = 0; c < 3; ++c) out[c] = v[c];
    return true;
  }
  bool need_attr(const XNode* n, const char* a, std::string& out) {
    const std::string* v = n->attr(a);
    if (!v) return fail("<" + n->name + "> needs the attribute " + a);
    out = *v;
    return true;
  }

  // LoadMesh_TetVolume (Serializer_XML.cpp:878-983)
  bool tet_volume(const XNode* n, std::vector<double>& V, std::vector<int32_t>& T, int* flipped) {
    std::string type;
    if (!need_attr(n, "type", type)) return false;
    if (type == "FILESURFACE")
      return fail("meshInit type FILESURFACE needs TetGen's mesher (MeshUtils::tetrahedralize); give a FILEVOLUME mesh");
    if (type != "FILEVOLUME") return fail("meshInit type " + type + " is not supported (FILEVOLUME is)");
    // the reference checks the attribute "path" and then reads the file name from "mesh"
    // (Serializer_XML.cpp:932-938); either names the file here, "mesh" first
    std::string p;
    if (!need_attr(n, "path", p)) return false;
    if (const std::string* mm = n->attr("mesh")) p = *mm;
    std::string e;
    if (!read_tetgen(resolve(p, dir), V, T, flipped, e)) return fail(e);
    // position, scale, rotation (degrees): V' = R S V + t
    double t[3] = {0, 0, 0}, sc[3] = {1, 1, 1}, rd[3] = {0, 0, 0};
    if (const XNode* c = n->child("position"))
      if (!vec3(c, t, "position")) return false;
    if (const XNode* c = n->child("scale"))
      if (!vec3(c, sc, "scale")) return false;
    if (const XNode* c = n->child("rotation")) {
      if (!vec3(c, rd, "rotation")) return false;
      for (double& d : rd) d = d * (3.14159265358979323846 / 180.0);  // MathUtils::degreesToRadians
    }
    const Mat3 R = euler(rd);
    const size_t np = V.size() / 3;
    for (size_t k = 0; k < np; ++k) {
      double s[3], o[3];
      for (int c = 0; c < 3; ++c) s[c] = sc[c] * V[3 * k + c];
      for (int r = 0; r < 3; ++r) o[r] = R.a[3 * r] * s[0] + R.a[3 * r + 1] * s[1] + R.a[3 * r + 2] * s[2] + t[r];
      for (int c = 0; c < 3; ++c) V[3 * k + c] = o[c];
    }
    return true;
  }

  // LoadDistribution (Serializer_XML.cpp:618-733): the objects of a CONSTANT or VARIABLE
  // distribution and each element's index into them.  An unknown type falls back to the
  // constant one, as the reference's last branch does.
  bool distribution(const XNode* n, int m, std::vector<const XNode*>& objs, std::vector<int>& idx) {
    std::string type;
    if (!need_attr(n, "type", type)) return false;
    objs = n->children(n->name.c_str());
    if (objs.empty()) return fail("<" + n->name + "> needs a <" + n->name + "> child");
    if (type == "SUBELEMENT") return fail("<" + n->name + "> SUBELEMENT distributions are not supported");
    if (type != "VARIABLE") {
      objs.resize(1);
      idx.assign(m, 0);
      return true;
    }
    if (const XNode* d = n->child("distribution")) {
      std::vector<double> v;
      if (!csv_numbers(d->text, v)) return fail("<distribution> of <" + n->name + "> is not a CSV vector");
      idx.resize(v.size());
      for (size_t k = 0; k < v.size(); ++k) idx[k] = (int)v[k];
    } else {
      idx.resize(objs.size());
      for (size_t k = 0; k < objs.size(); ++k) idx[k] = (int)k;
    }
    if ((int)idx.size() != m)
      return fail("<" + n->name + "> VARIABLE distribution maps " + std::to_string(idx.size()) + " elements, the mesh has " +
                  std::to_string(m));
    for (int k : idx)
      if (k < 0 || k >= (int)objs.size()) return fail("<" + n->name + "> distribution index out of range");
    return true;
  }

  // ParameterSet from <parameter name value> (Serializer_XML.cpp:577-616) with
  // InitLinearFromYoungPoisson / InitLinearFromLameParameters (ParameterSet.cpp:54-80)
  bool params(const XNode* n, double& lam, double& mu, double& rho) {
    std::map<std::string, double> p;
    for (const XNode* q : n->children("parameter")) {
      std::string nm, vv;
      if (!need_attr(q, "name", nm) || !need_attr(q, "value", vv)) return false;
      p[nm] = std::strtod(vv.c_str(), nullptr);
    }
    if (p.count("YOUNG") && p.count("POISSON") && p.count("DENSITY")) {
      const double E = p["YOUNG"], nu = p["POISSON"];
      const double t0 = 1 + nu, t1 = 1 - 2 * nu;
      lam = (E * nu) / (t0 * t1);
      mu = E / (2 * t0);
      rho = p["DENSITY"];
      return true;
    }
    if (p.count("LAME1") && p.count("LAME2") && p.count("DENSITY")) {
      lam = p["LAME1"];
      mu = p["LAME2"];
      rho = p["DENSITY"];
      return true;
    }
    return fail("<materialParam> needs YOUNG, POISSON and DENSITY, or LAME1, LAME2 and DENSITY");
  }

  bool simulable(const XNode* n, phx_scene_s& sc) {
    for (const char* c : {"meshInit", "discretization", "shapeFunction", "materialParam", "materialModel", "quadrature"})
      if (!n->child(c)) return fail(std::string("<") + n->name + "> needs a <" + c + "> child");
    std::string dis;
    if (!need_attr(n->child("discretization"), "type", dis)) return false;
    if (dis != "TET4") return fail("discretization " + dis + " is not supported (TET4 is)");
    std::vector<int32_t> T0;
    if (!tet_volume(n->child("meshInit"), sc.x_init, sc.T, &sc.flipped)) return false;
    sc.n = (int32_t)(sc.x_init.size() / 3);
    sc.m = (int32_t)(sc.T.size() / 4);
    if (const XNode* r = n->child("meshRest")) {
      int fr = 0;
      if (!tet_volume(r, sc.X0, T0, &fr)) return false;
      if (T0 != sc.T || sc.X0.size() != sc.x_init.size())
        return fail("meshRest must have the tetrahedra and points of meshInit");
    } else {
      sc.X0 = sc.x_init;
    }
    const int m = sc.m;
    std::vector<const XNode*> objs;
    std::vector<int> idx;
    // shape functions and quadratures: the Tet4 / Tet1 pair only
    if (!distribution(n->child("shapeFunction"), m, objs, idx)) return false;
    for (const XNode* o : objs) {
      std::string t;
      if (!need_attr(o, "type", t)) return false;
      if (t != "TET_LIN") return fail("shape function " + t + " is not supported (TET_LIN is)");
    }
    if (!distribution(n->child("quadrature"), m, objs, idx)) return false;
    for (const XNode* o : objs) {
      std::string t;
      if (!need_attr(o, "type", t)) return false;
      if (t != "TET_1") return fail("quadrature " + t + " is not supported (TET_1 is)");
    }
    // material models (Serializer_XML.cpp:528-575): CONH / STVK in 3D
    if (!distribution(n->child("materialModel"), m, objs, idx)) return false;
    std::vector<uint8_t> kinds;
    for (const XNode* o : objs) {
      std::string t, ds, db;
      if (!need_attr(o, "type", t) || !need_attr(o, "dimSpace", ds) || !need_attr(o, "dimBasis", db)) return false;
      if (ds != "3" || db != "3") return fail("material model " + t + " with dimSpace/dimBasis other than 3/3");
      if (t == "CONH") kinds.push_back(PHX_MODEL_CONH);
      else if (t == "STVK") kinds.push_back(PHX_MODEL_STVK);
      else return fail("material model " + t + " is not supported (CONH, STVK are)");
    }
    sc.model.resize(m);
    for (int e = 0; e < m; ++e) sc.model[e] = kinds[idx[e]];
    if (!distribution(n->child("materialParam"), m, objs, idx)) return false;
    std::vector<double> L, U, R;
    for (const XNode* o : objs) {
      double lam, mu, rho;
      if (!params(o, lam, mu, rho)) return false;
      L.push_back(lam);
      U.push_back(mu);
      R.push_back(rho);
    }
    sc.lame.resize(2 * (size_t)m);
    sc.rho.resize(m);
    for (int e = 0; e < m; ++e) {
      sc.lame[2 * e] = L[idx[e]];
      sc.lame[2 * e + 1] = U[idx[e]];
      sc.rho[e] = R[idx[e]];
    }
    sc.fixed.assign(3 * (size_t)sc.n, 0);
    return true;
  }

  bool problem(const XNode* n, phx_scene_s& sc) {
    std::string t;
    if (!need_attr(n, "type", t)) return false;
    if (t == "Static") {
      sc.dynamic = 0;
      return true;
    }
    if (t == "Dynamic") {
      std::string st;
      if (!need_attr(n, "step", st)) return false;
      sc.dynamic = 1;
      sc.dt = std::strtod(st.c_str(), nullptr);
      if (!(sc.dt > 0)) return fail("<problem> Dynamic needs a positive step");
      return true;
    }
    return fail("problem type " + t + " (Static, Dynamic)");
  }

  // LoadOptimSolver (Serializer_XML.cpp:1356-1505)
  bool solver(const XNode* n, phx_options& o) {
    if (const std::string* v = n->attr("maxIters")) o.num_max_iters = std::atoi(v->c_str());
    if (const std::string* v = n->attr("maxError")) o.tol_max_error = std::strtod(v->c_str(), nullptr);
    if (const std::string* v = n->attr("qpStep")) {
      if (*v == "Steepest") o.qp_solver = 0;
      else if (*v == "Newton") o.qp_solver = 1;
      else return fail("qpStep " + *v + " is not supported (Steepest, Newton are)");
    }
    if (const XNode* l = n->child("linear")) {
      if (const std::string* v = l->attr("type")) {
        // the device solves with preconditioned CG; EigenLDLT maps to it with the tolerance given
        if (*v != "EigenCG" && *v != "EigenLDLT") return fail("linear solver " + *v + " is not supported (EigenCG, EigenLDLT are)");
      }
      if (const std::string* v = l->attr("maxIters")) o.ls_num_max_iters = std::atoi(v->c_str());
      if (const std::string* v = l->attr("maxError")) o.ls_tol_max_error = std::strtod(v->c_str(), nullptr);
    }
    if (const XNode* l = n->child("lsearch")) {
      if (const std::string* v = l->attr("type")) {
        const char* names[] = {"None", "Simple", "Armijo", "WolfeWeak", "WolfeStrong"};
        int k = -1;
        for (int q = 0; q < 5; ++q)
          if (*v == names[q]) k = q;
        if (k < 0) return fail("line search " + *v + " (None, Simple, Armijo, WolfeWeak, WolfeStrong)");
        o.lsearch_type = k;
      }
      if (const std::string* v = l->attr("iters")) o.lsearch_num_try = std::atoi(v->c_str());
      if (const std::string* v = l->attr("alpha")) o.lsearch_alpha = std::strtod(v->c_str(), nullptr);
      if (const std::string* v = l->attr("wolfe1")) o.lsearch_wolfe1 = std::strtod(v->c_str(), nullptr);
      if (const std::string* v = l->attr("wolfe2")) o.lsearch_wolfe2 = std::strtod(v->c_str(), nullptr);
    }
    return true;
  }

  // LoadGeometryFilter (Serializer_XML.cpp:1758-1868), node selections
  bool selection(const XNode* n, const phx_scene_s& sc, std::vector<int32_t>& nodes) {
    std::string t;
    if (!need_attr(n, "type", t)) return false;
    nodes.clear();
    if (t == "AllNodes") {
      for (int v = 0; v < sc.n; ++v) nodes.push_back(v);
      return true;
    }
    if (t == "IndexNodes") {
      std::vector<double> v;
      if (!n->child("indices") || !csv_numbers(n->child("indices")->text, v)) return fail("IndexNodes needs <indices>");
      for (double d : v) {
        const int k = (int)d;
        if (k < 0 || k >= sc.n) return fail("IndexNodes: index out of range");
        nodes.push_back(k);
      }
      return true;
    }
    if (t == "BoxNodes") {
      double lo[3], hi[3];
      std::string field;
      if (!vec3(n->child("minCorner"), lo, "minCorner") || !vec3(n->child("maxCorner"), hi, "maxCorner")) return false;
      if (!need_attr(n, "field", field)) return false;
      const std::vector<double>* F = nullptr;
      std::vector<double> zero;
      if (field == "Pos0") F = &sc.X0;
      else if (field == "PosX") F = &sc.x_init;
      else if (field == "VelX") {
        zero.assign(sc.x_init.size(), 0.0);
        F = &zero;
      } else {
        return fail("BoxNodes field " + field + " (Pos0, PosX, VelX)");
      }
      // GeometryFilter_BoxNodes::Filter (GeometryFilters.h:207-227): inside, bounds included
      for (int v = 0; v < sc.n; ++v) {
        const double* p = &(*F)[3 * (size_t)v];
        if (p[0] >= lo[0] && p[0] <= hi[0] && p[1] >= lo[1] && p[1] <= hi[1] && p[2] >= lo[2] && p[2] <= hi[2])
          nodes.push_back(v);
      }
      return true;
    }
    if (t == "BoundaryNodes") {
      // nodes of the faces that belong to one tetrahedron only
      std::map<std::array<int32_t, 3>, int> faces;
      static const int F4[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
      for (int e = 0; e < sc.m; ++e)
        for (auto& f : F4) {
          std::array<int32_t, 3> k = {sc.T[4 * e + f[0]], sc.T[4 * e + f[1]], sc.T[4 * e + f[2]]};
          std::sort(k.begin(), k.end());
          faces[k]++;
        }
      std::vector<char> on(sc.n, 0);
      for (auto& kv : faces)
        if (kv.second == 1)
          for (int32_t v : kv.first) on[v] = 1;
      for (int v = 0; v < sc.n; ++v)
        if (on[v]) nodes.push_back(v);
      return true;
    }
    return fail("selection " + t + " is not supported for FixPosition (AllNodes, BoundaryNodes, IndexNodes, BoxNodes)");
  }

  // LoadBoundary (Serializer_XML.cpp:1507-1647)
  bool boundary(const XNode* n, phx_scene_s& sc) {
    std::vector<char> taken(sc.n, 0);
    for (const XNode* bc : n->children("bc")) {
      std::string t;
      if (!need_attr(bc, "type", t)) return false;
      int stages = 1;
      if (const std::string* v = bc->attr("numStep")) stages = std::atoi(v->c_str());
      if (stages < 1) return fail("numStep must be at least 1");
      sc.num_stages = std::max(sc.num_stages, stages);
      if (t == "Gravity") {
        double g[3] = {0.0, -9.8, 0.0};  // the reference's default acceleration
        if (const XNode* c = bc->child("gravity"))
          if (!vec3(c, g, "gravity")) return false;
        for (int c = 0; c < 3; ++c) sc.gravity[c] = g[c];
        continue;
      }
      if (t == "FixPosition") {
        std::string so;
        if (!need_attr(bc, "soft", so)) return false;
        if (!bc->child("selection")) return fail("FixPosition needs a <selection>");
        const bool soft = so == "true" || so == "1";
        std::vector<int32_t> nodes;
        if (!selection(bc->child("selection"), sc, nodes)) return false;
        for (int32_t v : nodes) {
          if (soft) {
            // BC_FixDoF soft mode with its default stiffness kAini = kAend = 1e9 (BC_FixDoF.h:27-32),
            // the target the node's position when the scene is loaded
            if (sc.soft_k.empty()) {
              sc.soft_k.assign(sc.n, 0.0);
              sc.soft_t = sc.x_init;
            }
            sc.soft_k[v] = 1e9;
          } else {
            for (int c = 0; c < 3; ++c) sc.fixed[3 * (size_t)v + c] = 1;
          }
        }
        if (const XNode* a = bc->child("animation")) {
          std::string at;
          if (!need_attr(a, "type", at)) return false;
          if (at != "Transform3D") return fail("animation " + at + " is not supported (Transform3D is)");
          // VectorAnimator_LerpT3D(vT, vR, vS) (VectorAnimators.h:109-121): its 4x4 holds R S and
          // t, and Evaluate adds a times it to the identity (:135-145).  The rotation is read in
          // radians here (LoadVector3D, Serializer_XML.cpp:1658-1671), unlike a mesh's degrees.
          double tv[3] = {0, 0, 0}, rv[3] = {0, 0, 0}, sv[3] = {1, 1, 1};
          if (a->child("position") && !vec3(a->child("position"), tv, "position")) return false;
          if (a->child("rotation") && !vec3(a->child("rotation"), rv, "rotation")) return false;
          if (a->child("scale") && !vec3(a->child("scale"), sv, "scale")) return false;
          const Mat3 Rm = euler(rv);
          phx_scene_s::Group G;
          G.g.num_stages = stages;
          G.g.soft = soft ? 1 : 0;
          G.g.k_start = G.g.k_end = 1e9;
          for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) G.g.move[3 * r + c] = Rm.a[3 * r + c] * sv[c];
          for (int c = 0; c < 3; ++c) G.g.shift[c] = tv[c];
          for (int32_t v : nodes) {
            if (taken[v]) return fail("a node is moved by two animated FixPosition conditions");
            taken[v] = 1;
          }
          G.nodes = nodes;
          sc.groups.push_back(std::move(G));
        }
        continue;
      }
      if (t == "CollPlane") return fail("CollPlane (contact) is outside the tet-FEM Newton path");
      if (t == "Force" || t == "AlignFace")
        return fail("bc type " + t + ": the reference's loader creates no condition for it (Serializer_XML.cpp:1592-1632)");
      return fail("bc type " + t + " (Gravity, FixPosition)");
    }
    return true;
  }

  bool scene(const XNode& root, phx_scene_s& sc) {
    const XNode* sim = root.child("simulable");
    if (!sim) return fail("the scene needs a <simulable> element (the VolumeFEM model)");
    if (const std::string* t = sim->attr("type"))
      if (*t != "VolumeFEM") return fail("simulable type " + *t + " is not supported (VolumeFEM is)");
    if (!simulable(sim, sc)) return false;
    phx_default_options(&sc.opts);
    if (const XNode* p = root.child("problem"))
      if (!problem(p, sc)) return false;
    if (const XNode* s = root.child("solver"))
      if (!solver(s, sc.opts)) return false;
    if (const XNode* b = root.child("boundary"))
      if (!boundary(b, sc)) return false;
    return true;
  }
};

int fail_scene(int code, const std::string& m) { return phx::set_last_error(code, m); }

}  // namespace

extern "C" {

int phx_scene_load(const char* path, phx_scene* out) {
  if (!path || !out) return fail_scene(PHX_EINVAL, "NULL argument");
  *out = nullptr;
  try {
    std::string src;
    if (!read_file(path, src)) return fail_scene(PHX_EINVAL, std::string("cannot read ") + path);
    XNode root;
    XParser xp(src);
    if (!xp.document(root)) return fail_scene(PHX_EINVAL, std::string(path) + ": " + xp.err);
    std::unique_ptr<phx_scene_s> sc(new phx_scene_s());
    Loader L;
    L.dir = dir_of(path);
    if (!L.scene(root, *sc)) return fail_scene(PHX_EINVAL, std::string(path) + ": " + L.err);
    for (auto& G : sc->groups) {
      G.g.num_nodes = (int32_t)G.nodes.size();
      G.g.nodes = G.nodes.data();
    }
    *out = sc.release();
    return PHX_OK;
  } catch (const std::bad_alloc&) {
    return fail_scene(PHX_ENOMEM, "out of host memory reading the scene");
  } catch (...) {
    return fail_scene(PHX_EINVAL, "unexpected error reading the scene");
  }
}

int phx_scene_destroy(phx_scene sc) {
  delete sc;
  return PHX_OK;
}

int phx_scene_info(phx_scene sc, int32_t* num_nodes, int32_t* num_tets, int32_t* dynamic, double* dt,
                   int32_t* num_groups, int32_t* num_stages, int32_t* reoriented) {
  if (!sc) return fail_scene(PHX_EINVAL, "scene is NULL");
  if (num_nodes) *num_nodes = sc->n;
  if (num_tets) *num_tets = sc->m;
  if (dynamic) *dynamic = sc->dynamic;
  if (dt) *dt = sc->dt;
  if (num_groups) *num_groups = (int32_t)sc->groups.size();
  if (num_stages) *num_stages = sc->num_stages;
  if (reoriented) *reoriented = sc->flipped;
  return PHX_OK;
}

int phx_scene_mesh(phx_scene sc, phx_mesh* mesh, double* x_init) {
  if (!sc || !mesh) return fail_scene(PHX_EINVAL, "NULL argument");
  std::memset(mesh, 0, sizeof(*mesh));
  mesh->num_nodes = sc->n;
  mesh->num_tets = sc->m;
  mesh->X0 = sc->X0.data();
  mesh->tets = sc->T.data();
  mesh->lame = sc->lame.data();
  mesh->rho = sc->rho.data();
  mesh->model = sc->model.data();
  mesh->fixed = sc->fixed.data();
  mesh->force = nullptr;
  for (int c = 0; c < 3; ++c) mesh->gravity[c] = sc->gravity[c];
  mesh->soft_k = sc->soft_k.empty() ? nullptr : sc->soft_k.data();
  mesh->soft_target = sc->soft_k.empty() ? nullptr : sc->soft_t.data();
  if (x_init) std::copy(sc->x_init.begin(), sc->x_init.end(), x_init);
  return PHX_OK;
}

int phx_scene_options(phx_scene sc, phx_options* opts) {
  if (!sc || !opts) return fail_scene(PHX_EINVAL, "NULL argument");
  *opts = sc->opts;
  return PHX_OK;
}

int phx_scene_staging(phx_scene sc, phx_stage_group* groups, int32_t cap) {
  if (!sc) return fail_scene(PHX_EINVAL, "scene is NULL");
  const int32_t n = (int32_t)sc->groups.size();
  if (groups)
    for (int32_t k = 0; k < std::min(n, cap); ++k) groups[k] = sc->groups[k].g;
  return n;
}

int phx_scene_instance(phx_context ctx, phx_scene sc, phx_instance* out) {
  if (!ctx || !sc || !out) return fail_scene(PHX_EINVAL, "NULL argument");
  *out = nullptr;
  phx_mesh mesh;
  int rc = phx_scene_mesh(sc, &mesh, nullptr);
  if (rc) return rc;
  phx_instance inst = nullptr;
  if ((rc = phx_instance_create(ctx, &mesh, &inst))) return rc;
  // the model starts at meshInit (Position_X); targets and staging start from there too
  if ((rc = phx_instance_set_positions(inst, sc->x_init.data()))) {
    phx_instance_destroy(inst);
    return rc;
  }
  if (!sc->groups.empty() || sc->num_stages > 1) {
    std::vector<phx_stage_group> gs;
    for (auto& G : sc->groups) gs.push_back(G.g);
    if ((rc = phx_instance_set_staging(inst, (int32_t)gs.size(), gs.data(), sc->num_stages))) {
      phx_instance_destroy(inst);
      return rc;
    }
  }
  *out = inst;
  return PHX_OK;
}

}  // extern "C"
