// .ori scene loader: XML + OBJ -> flat HostScene.
//
// Mirrors the reference parser's semantics (src/util/parser.cpp:45-471,
// src/util/strutil.cpp, src/core/triangle.cpp:8-58,137-151,
// src/core/transform.cpp) with its own small XML reader, so a scene file
// that renders in the reference loads here into the same primitives,
// materials, lights and camera, in the same order:
//   * primitives in <Model> order, triangles in file order, vertices and
//     normals baked into world space with the model transform;
//   * named materials: the first definition of a name wins;
//   * lights: one area light per emissive triangle (model order), then
//     <Light> elements, then <Envmap> elements.
// Differences, all deliberate: the resource directory is resolved against
// the scene file's directory (the reference prefixes the executable path,
// src/util/envvariable.cpp:37-40); named materials and stored transforms
// are per file rather than process-wide; an image texture's file name, which
// the reference opens relative to the working directory
// (src/util/parser.cpp:438-443), is looked up in the resource directory, then
// the scene's directory, then the working directory; features outside the
// path tracer (SPD files, named metals, the pseudo-random sampler) are
// reported as ORION_ERR_UNSUPPORTED instead of being loaded.
#include "scene_host.h"
#include "image_io.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <thread>
#include <utility>
#include <vector>

namespace orion_gb300 {

// ------------------------------------------------------------------ math

float radians_f(float deg) { return deg * static_cast<float>(0.01745329251994329576923690768489); }
float degrees_f(float rad) { return rad * static_cast<float>(57.295779513082320876798154814105); }

Mat4 Mat4::identity() { return make(1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1); }

Mat4 Mat4::make(float t00, float t01, float t02, float t03, float t10, float t11, float t12, float t13, float t20,
                float t21, float t22, float t23, float t30, float t31, float t32, float t33) {
  Mat4 r;
  float v[16] = {t00, t01, t02, t03, t10, t11, t12, t13, t20, t21, t22, t23, t30, t31, t32, t33};
  std::memcpy(r.m, v, sizeof(v));
  return r;
}

Mat4 Mat4::operator*(const Mat4& b) const {
  Mat4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      r.m[i][j] = m[i][0] * b.m[0][j] + m[i][1] * b.m[1][j] + m[i][2] * b.m[2][j] + m[i][3] * b.m[3][j];
  return r;
}

Mat4 Mat4::transposed() const {
  Mat4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r.m[i][j] = m[j][i];
  return r;
}

// Gauss-Jordan elimination with full pivoting (the classic gaussj scheme the
// reference uses at src/core/transform.cpp:44-100): pivot search over
// unused rows/columns with >=, row swap onto the diagonal, scale, eliminate,
// then undo the column permutation in reverse order.
Mat4 Mat4::inverse() const {
  int indxc[4], indxr[4];
  int ipiv[4] = {0, 0, 0, 0};
  float a[4][4];
  std::memcpy(a, m, sizeof(a));
  for (int i = 0; i < 4; ++i) {
    int irow = 0, icol = 0;
    float big = 0.f;
    for (int j = 0; j < 4; ++j) {
      if (ipiv[j] == 1) continue;
      for (int k = 0; k < 4; ++k) {
        if (ipiv[k] == 0 && std::fabs(a[j][k]) >= big) {
          big = std::fabs(a[j][k]);
          irow = j;
          icol = k;
        }
      }
    }
    ++ipiv[icol];
    if (irow != icol)
      for (int k = 0; k < 4; ++k) std::swap(a[irow][k], a[icol][k]);
    indxr[i] = irow;
    indxc[i] = icol;
    float pivinv = 1.f / a[icol][icol];
    a[icol][icol] = 1.f;
    for (int j = 0; j < 4; ++j) a[icol][j] *= pivinv;
    for (int j = 0; j < 4; ++j) {
      if (j == icol) continue;
      float save = a[j][icol];
      a[j][icol] = 0.f;
      for (int k = 0; k < 4; ++k) a[j][k] -= a[icol][k] * save;
    }
  }
  for (int j = 3; j >= 0; --j)
    if (indxr[j] != indxc[j])
      for (int k = 0; k < 4; ++k) std::swap(a[k][indxr[j]], a[k][indxc[j]]);
  Mat4 r;
  std::memcpy(r.m, a, sizeof(a));
  return r;
}

void Xform::point(const float in[3], float out[3]) const {
  float x = in[0], y = in[1], z = in[2];
  float xp = m.m[0][0] * x + m.m[0][1] * y + m.m[0][2] * z + m.m[0][3];
  float yp = m.m[1][0] * x + m.m[1][1] * y + m.m[1][2] * z + m.m[1][3];
  float zp = m.m[2][0] * x + m.m[2][1] * y + m.m[2][2] * z + m.m[2][3];
  float wp = m.m[3][0] * x + m.m[3][1] * y + m.m[3][2] * z + m.m[3][3];
  if (wp == 1.f) {
    out[0] = xp;
    out[1] = yp;
    out[2] = zp;
  } else {
    float inv = 1.f / wp;
    out[0] = inv * xp;
    out[1] = inv * yp;
    out[2] = inv * zp;
  }
}

void Xform::vector(const float in[3], float out[3]) const {
  float x = in[0], y = in[1], z = in[2];
  out[0] = m.m[0][0] * x + m.m[0][1] * y + m.m[0][2] * z;
  out[1] = m.m[1][0] * x + m.m[1][1] * y + m.m[1][2] * z;
  out[2] = m.m[2][0] * x + m.m[2][1] * y + m.m[2][2] * z;
}

void Xform::normal(const float in[3], float out[3]) const {
  float x = in[0], y = in[1], z = in[2];
  out[0] = minv.m[0][0] * x + minv.m[1][0] * y + minv.m[2][0] * z;
  out[1] = minv.m[0][1] * x + minv.m[1][1] * y + minv.m[2][1] * z;
  out[2] = minv.m[0][2] * x + minv.m[1][2] * y + minv.m[2][2] * z;
}

Xform Xform::translate(float x, float y, float z) {
  return Xform(Mat4::make(1, 0, 0, x, 0, 1, 0, y, 0, 0, 1, z, 0, 0, 0, 1),
               Mat4::make(1, 0, 0, -x, 0, 1, 0, -y, 0, 0, 1, -z, 0, 0, 0, 1));
}

Xform Xform::scale(float x, float y, float z) {
  return Xform(Mat4::make(x, 0, 0, 0, 0, y, 0, 0, 0, 0, z, 0, 0, 0, 0, 1),
               Mat4::make(1 / x, 0, 0, 0, 0, 1 / y, 0, 0, 0, 0, 1 / z, 0, 0, 0, 0, 1));
}

namespace {
void v_normalize(const float in[3], float out[3]) {
  float len = std::sqrt(in[0] * in[0] + in[1] * in[1] + in[2] * in[2]);
  float inv = 1.f / len;
  out[0] = in[0] * inv;
  out[1] = in[1] * inv;
  out[2] = in[2] * inv;
}
void v_cross(const float a[3], const float b[3], float out[3]) {
  float r0 = a[1] * b[2] - a[2] * b[1];
  float r1 = a[2] * b[0] - a[0] * b[2];
  float r2 = a[0] * b[1] - a[1] * b[0];
  out[0] = r0;
  out[1] = r1;
  out[2] = r2;
}
float v_dot(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
}  // namespace

// Rodrigues rotation about a normalised axis (src/core/transform.cpp:170-196).
Xform Xform::rotate(float theta, const float axis[3]) {
  float a[3];
  v_normalize(axis, a);
  float s = std::sin(radians_f(theta));
  float c = std::cos(radians_f(theta));
  Mat4 r = Mat4::identity();
  r.m[0][0] = a[0] * a[0] + (1 - a[0] * a[0]) * c;
  r.m[0][1] = a[0] * a[1] * (1 - c) - a[2] * s;
  r.m[0][2] = a[0] * a[2] * (1 - c) + a[1] * s;
  r.m[0][3] = 0;
  r.m[1][0] = a[0] * a[1] * (1 - c) + a[2] * s;
  r.m[1][1] = a[1] * a[1] + (1 - a[1] * a[1]) * c;
  r.m[1][2] = a[1] * a[2] * (1 - c) - a[0] * s;
  r.m[1][3] = 0;
  r.m[2][0] = a[0] * a[2] * (1 - c) - a[1] * s;
  r.m[2][1] = a[1] * a[2] * (1 - c) + a[0] * s;
  r.m[2][2] = a[2] * a[2] + (1 - a[2] * a[2]) * c;
  r.m[2][3] = 0;
  return Xform(r, r.transposed());
}

// World-from-camera for a camera at `pos` looking at `look`
// (src/core/transform.cpp:197-217): the view matrix is built directly and
// inverted by Gauss-Jordan.
Xform Xform::look_at(const float pos[3], const float look[3], const float up[3]) {
  float d[3] = {look[0] - pos[0], look[1] - pos[1], look[2] - pos[2]};
  float f[3], s[3], u[3], t[3];
  v_normalize(d, f);
  v_cross(f, up, t);
  v_normalize(t, s);
  v_cross(s, f, u);
  Mat4 r = Mat4::identity();
  r.m[0][0] = s[0];
  r.m[0][1] = s[1];
  r.m[0][2] = s[2];
  r.m[1][0] = u[0];
  r.m[1][1] = u[1];
  r.m[1][2] = u[2];
  r.m[2][0] = -f[0];
  r.m[2][1] = -f[1];
  r.m[2][2] = -f[2];
  r.m[0][3] = -v_dot(s, pos);
  r.m[1][3] = -v_dot(u, pos);
  r.m[2][3] = v_dot(f, pos);
  return Xform(r.inverse(), r);
}

// ------------------------------------------------------------ xml reader

namespace {

struct XmlNode {
  std::string name;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::vector<std::unique_ptr<XmlNode>> children;

  const char* attr(const char* key) const {
    for (const auto& a : attrs)
      if (a.first == key) return a.second.c_str();
    return nullptr;
  }
  const XmlNode* child(const char* nm) const {
    for (const auto& c : children)
      if (c->name == nm) return c.get();
    return nullptr;
  }
  std::vector<const XmlNode*> all(const char* nm) const {
    std::vector<const XmlNode*> r;
    for (const auto& c : children)
      if (c->name == nm) r.push_back(c.get());
    return r;
  }
};

class XmlReader {
 public:
  explicit XmlReader(const std::string& s) : s_(s) {}

  std::unique_ptr<XmlNode> parse_document(std::string* err) {
    std::unique_ptr<XmlNode> root;
    while (true) {
      skip_misc();
      if (pos_ >= s_.size()) break;
      if (s_[pos_] != '<') return fail(err, "text outside the root element");
      auto el = parse_element(err);
      if (!el) return nullptr;
      if (!root) root = std::move(el);
    }
    if (!root) return fail(err, "no root element");
    return root;
  }

 private:
  const std::string& s_;
  size_t pos_ = 0;

  std::unique_ptr<XmlNode> fail(std::string* err, const std::string& msg) {
    size_t line = 1;
    for (size_t i = 0; i < pos_ && i < s_.size(); ++i) line += s_[i] == '\n';
    *err = "XML line " + std::to_string(line) + ": " + msg;
    return nullptr;
  }
  bool starts(const char* p) const { return s_.compare(pos_, std::strlen(p), p) == 0; }
  void skip_ws() {
    while (pos_ < s_.size() && std::isspace((unsigned char)s_[pos_])) ++pos_;
  }
  // Whitespace, comments, <?...?> declarations and <!...> directives.
  void skip_misc() {
    while (true) {
      skip_ws();
      if (starts("<!--")) {
        size_t e = s_.find("-->", pos_ + 4);
        pos_ = e == std::string::npos ? s_.size() : e + 3;
      } else if (starts("<?")) {
        size_t e = s_.find("?>", pos_ + 2);
        pos_ = e == std::string::npos ? s_.size() : e + 2;
      } else if (starts("<!")) {
        size_t e = s_.find('>', pos_ + 2);
        pos_ = e == std::string::npos ? s_.size() : e + 1;
      } else {
        return;
      }
    }
  }
  std::string name() {
    size_t b = pos_;
    while (pos_ < s_.size() && !std::isspace((unsigned char)s_[pos_]) && s_[pos_] != '>' && s_[pos_] != '/' &&
           s_[pos_] != '=')
      ++pos_;
    return s_.substr(b, pos_ - b);
  }
  static std::string decode(const std::string& v) {
    std::string r;
    for (size_t i = 0; i < v.size(); ++i) {
      if (v[i] == '&') {
        static const char* ents[][2] = {{"&amp;", "&"}, {"&lt;", "<"}, {"&gt;", ">"}, {"&quot;", "\""}, {"&apos;", "'"}};
        bool hit = false;
        for (auto& e : ents)
          if (v.compare(i, std::strlen(e[0]), e[0]) == 0) {
            r += e[1];
            i += std::strlen(e[0]) - 1;
            hit = true;
            break;
          }
        if (!hit) r += v[i];
      } else {
        r += v[i];
      }
    }
    return r;
  }
  std::unique_ptr<XmlNode> parse_element(std::string* err) {
    ++pos_;  // '<'
    auto node = std::make_unique<XmlNode>();
    node->name = name();
    if (node->name.empty()) return fail(err, "empty element name");
    while (true) {
      skip_ws();
      if (pos_ >= s_.size()) return fail(err, "unterminated tag <" + node->name + ">");
      if (starts("/>")) {
        pos_ += 2;
        return node;
      }
      if (s_[pos_] == '>') {
        ++pos_;
        break;
      }
      std::string key = name();
      if (key.empty()) return fail(err, "bad attribute in <" + node->name + ">");
      skip_ws();
      if (pos_ >= s_.size() || s_[pos_] != '=') return fail(err, "attribute '" + key + "' without value");
      ++pos_;
      skip_ws();
      if (pos_ >= s_.size() || (s_[pos_] != '"' && s_[pos_] != '\'')) return fail(err, "unquoted attribute " + key);
      char q = s_[pos_++];
      size_t e = s_.find(q, pos_);
      if (e == std::string::npos) return fail(err, "unterminated attribute " + key);
      node->attrs.emplace_back(key, decode(s_.substr(pos_, e - pos_)));
      pos_ = e + 1;
    }
    // content
    while (true) {
      size_t lt = s_.find('<', pos_);
      if (lt == std::string::npos) return fail(err, "missing </" + node->name + ">");
      pos_ = lt;
      if (starts("<!--") || starts("<?") || (starts("<!") && !starts("<![CDATA["))) {
        skip_misc();
        continue;
      }
      if (starts("<![CDATA[")) {
        size_t e = s_.find("]]>", pos_);
        pos_ = e == std::string::npos ? s_.size() : e + 3;
        continue;
      }
      if (starts("</")) {
        pos_ += 2;
        std::string nm = name();
        skip_ws();
        if (nm != node->name) return fail(err, "</" + nm + "> closes <" + node->name + ">");
        if (pos_ >= s_.size() || s_[pos_] != '>') return fail(err, "bad closing tag");
        ++pos_;
        return node;
      }
      auto c = parse_element(err);
      if (!c) return nullptr;
      node->children.push_back(std::move(c));
    }
  }
};

// ------------------------------------------------------ string parsing

std::string trim(std::string s) {
  size_t b = s.find_first_not_of(' ');
  if (b == std::string::npos) return std::string();
  size_t e = s.find_last_not_of(' ');
  return s.substr(b, e - b + 1);
}

std::vector<std::string> split_commas(const std::string& s) {
  std::vector<std::string> r;
  size_t last = 0;
  while (true) {
    size_t i = s.find(',', last);
    if (i == std::string::npos) {
      r.push_back(s.substr(last));
      break;
    }
    r.push_back(s.substr(last, i - last));
    last = i + 1;
  }
  return r;
}

float parse_float(const std::string& s) { return static_cast<float>(std::atof(s.c_str())); }
int parse_int(const std::string& s) { return std::atoi(s.c_str()); }

struct ParamMap {  // first definition of a key wins (src/util/param.h:38-42)
  std::map<std::string, std::string> kv;
  bool has(const std::string& k) const { return kv.count(k) != 0; }
  const std::string& get(const std::string& k) const {
    static const std::string empty;
    auto it = kv.find(k);
    return it == kv.end() ? empty : it->second;
  }
};

ParamMap params_of(const XmlNode* n) {
  ParamMap pm;
  if (!n) return pm;
  for (const XmlNode* p : n->all("Param"))
    for (const auto& a : p->attrs) pm.kv.insert(a);
  return pm;
}

std::vector<std::pair<std::string, std::string>> param_list(const XmlNode* n) {
  std::vector<std::pair<std::string, std::string>> r;
  if (!n) return r;
  for (const XmlNode* p : n->all("Param"))
    for (const auto& a : p->attrs) r.push_back(a);
  return r;
}

struct LoadError {
  int code;
  std::string msg;
};

[[noreturn]] void raise(int code, const std::string& msg) { throw LoadError{code, msg}; }

void parse_vec3(const std::string& s, float out[3], const char* what) {
  auto v = split_commas(s);
  if (v.size() < 3) raise(ORION_ERR_PARSE, std::string("need 3 numbers for ") + what + ": '" + s + "'");
  for (int i = 0; i < 3; ++i) out[i] = parse_float(v[i]);
}

void parse_spectrum(const std::string& s, float out[3]) {
  auto v = split_commas(s);
  if (v.size() < 3) {
    out[0] = out[1] = out[2] = parse_float(v[0]);
    return;
  }
  for (int i = 0; i < 3; ++i) out[i] = parse_float(v[i]);
}

// createTransform (src/core/transform.cpp:218-250): each parameter is
// applied on the left of the accumulated transform, in document order.
Xform make_transform(const XmlNode* tnode, std::vector<Xform>* reuse) {
  Xform t;
  for (const auto& kv : param_list(tnode)) {
    const std::string& k = kv.first;
    const std::string& v = kv.second;
    if (k == "store") {
      int pos = parse_int(v);
      if (pos < 0 || pos >= (int)reuse->size()) raise(ORION_ERR_PARSE, "transform store slot out of range");
      (*reuse)[pos] = t;
    } else if (k == "reuse") {
      int pos = parse_int(v);
      if (pos < 0 || pos >= (int)reuse->size()) raise(ORION_ERR_PARSE, "transform reuse slot out of range");
      t = (*reuse)[pos] * t;
    } else if (k == "scale") {
      float s[3];
      parse_vec3(v, s, "scale");
      t = Xform::scale(s[0], s[1], s[2]) * t;
    } else if (k == "rotate") {
      auto p = split_commas(v);
      if (p.size() <= 3) raise(ORION_ERR_PARSE, "rotate needs axis and angle");
      float axis[3] = {parse_float(p[0]), parse_float(p[1]), parse_float(p[2])};
      t = Xform::rotate(parse_float(p[3]), axis) * t;
    } else if (k == "translate") {
      float s[3];
      parse_vec3(v, s, "translate");
      t = Xform::translate(s[0], s[1], s[2]) * t;
    } else if (k == "lookat") {
      auto p = split_commas(v);
      if (p.size() < 9) raise(ORION_ERR_PARSE, "lookat needs 9 numbers");
      float a[3], b[3], c[3];
      for (int i = 0; i < 3; ++i) {
        a[i] = parse_float(p[i]);
        b[i] = parse_float(p[3 + i]);
        c[i] = parse_float(p[6 + i]);
      }
      t = Xform::look_at(a, b, c) * t;
    }
  }
  return t;
}

// ------------------------------------------------------------- obj mesh

struct CornerMesh {  // de-indexed: 3 corners per triangle
  std::vector<float> p, n, uv;
  int num_tris = 0;
};

bool read_file(const std::string& path, std::string* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out->resize(n > 0 ? (size_t)n : 0);
  const bool ok = n >= 0 && std::fread(&(*out)[0], 1, out->size(), f) == out->size();
  std::fclose(f);
  return ok;
}

// Wavefront OBJ as the reference reads it through tiny_obj_loader
// (src/core/triangle.cpp:8-58): polygons fan-triangulated, positions and
// normals required per corner, texture coordinates optional (0 if absent).
//
// The file is parsed in line-aligned pieces on several threads; each piece
// keeps its own vertex arrays and face corners, which are then joined in file
// order (relative indices resolved against the vertices read before them), so
// the triangles and their order are those of a sequential read.
namespace obj {

struct Corner {
  long v, t, n;  // as written: 1-based, negative = relative, 0 = absent
};

struct Piece {
  const char* begin;
  const char* end;
  std::vector<float> v, vn, vt;
  std::vector<Corner> corners;
  std::vector<int> face_first;   // first corner of each face
  std::vector<int> face_line;    // line of each face within the piece
  std::vector<int> face_counts;  // v, vt, vn counts in the piece when the face was read
  int lines = 0;
  int64_t tris = 0;
  std::string error;  // "line: message"
};

void parse_piece(Piece& pc) {
  const char* s = pc.begin;
  while (s < pc.end) {
    const char* eol = (const char*)std::memchr(s, '\n', pc.end - s);
    if (!eol) eol = pc.end;
    ++pc.lines;
    const char* p = s;
    while (p < eol && (*p == ' ' || *p == '\t')) ++p;
    if (p + 1 < eol && p[0] == 'v' && (p[1] == ' ' || p[1] == '\t')) {
      char* q;
      float x = std::strtof(p + 2, &q);
      float y = std::strtof(q, &q);
      float z = std::strtof(q, &q);
      pc.v.insert(pc.v.end(), {x, y, z});
    } else if (p + 2 < eol && p[0] == 'v' && p[1] == 'n' && (p[2] == ' ' || p[2] == '\t')) {
      char* q;
      float x = std::strtof(p + 3, &q);
      float y = std::strtof(q, &q);
      float z = std::strtof(q, &q);
      pc.vn.insert(pc.vn.end(), {x, y, z});
    } else if (p + 2 < eol && p[0] == 'v' && p[1] == 't' && (p[2] == ' ' || p[2] == '\t')) {
      char* q;
      float x = std::strtof(p + 3, &q);
      float y = std::strtof(q, &q);
      pc.vt.insert(pc.vt.end(), {x, y});
    } else if (p + 1 < eol && p[0] == 'f' && (p[1] == ' ' || p[1] == '\t')) {
      const int first = (int)pc.corners.size();
      const char* q = p + 2;
      while (q < eol) {
        while (q < eol && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q >= eol) break;
        char* r;
        long a = std::strtol(q, &r, 10);
        long b = 0, c = 0;
        if (r == q) {
          pc.error = std::to_string(pc.lines) + ": bad face";
          return;
        }
        q = r;
        if (q < eol && *q == '/') {
          ++q;
          if (q < eol && *q != '/') {
            b = std::strtol(q, &r, 10);
            q = r;
          }
          if (q < eol && *q == '/') {
            ++q;
            c = std::strtol(q, &r, 10);
            q = r;
          }
        }
        pc.corners.push_back(Corner{a, b, c});
        while (q < eol && *q != ' ' && *q != '\t') ++q;
      }
      const int nc = (int)pc.corners.size() - first;
      if (nc < 3) {
        pc.error = std::to_string(pc.lines) + ": face with < 3 corners";
        return;
      }
      pc.face_first.push_back(first);
      pc.face_line.push_back(pc.lines);
      pc.face_counts.insert(pc.face_counts.end(),
                            {(int)(pc.v.size() / 3), (int)(pc.vt.size() / 2), (int)(pc.vn.size() / 3)});
      pc.tris += nc - 2;
    }
    s = eol + 1;
  }
}

}  // namespace obj

void load_obj(const std::string& path, CornerMesh* out) {
  std::string text;
  if (!read_file(path, &text)) raise(ORION_ERR_IO, "cannot read mesh " + path);
  const char* s = text.data();
  const char* end = s + text.size();
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int npieces = text.size() < (1u << 20) ? 1 : std::min(4 * hw, (int)(text.size() >> 18));
  std::vector<obj::Piece> pcs(npieces);
  const char* cut = s;
  for (int i = 0; i < npieces; ++i) {  // line-aligned pieces
    const char* e = i + 1 == npieces ? end : s + (text.size() * (size_t)(i + 1)) / npieces;
    if (e < cut) e = cut;
    const char* nl = e < end ? (const char*)std::memchr(e, '\n', end - e) : nullptr;
    e = (i + 1 == npieces || !nl) ? end : nl + 1;
    pcs[i].begin = cut;
    pcs[i].end = e;
    cut = e;
  }
  auto for_pieces = [&](auto f) {
    std::vector<std::thread> th;
    std::atomic<int> next{0};
    const int nt = std::min(hw, npieces);
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&] {
        for (int i; (i = next.fetch_add(1)) < npieces;) f(i);
      });
    for (auto& x : th) x.join();
  };
  for_pieces([&](int i) { obj::parse_piece(pcs[i]); });
  // Join: vertex arrays in file order, global line numbers, triangle offsets.
  std::vector<int64_t> v0(npieces), t0(npieces), n0(npieces), line0(npieces), tri0(npieces);
  std::vector<float> v, vn, vt;
  int64_t lines = 0, tris = 0;
  for (int i = 0; i < npieces; ++i) {
    const obj::Piece& pc = pcs[i];
    if (!pc.error.empty()) {
      const size_t colon = pc.error.find(':');
      raise(ORION_ERR_PARSE, path + ":" + std::to_string(lines + std::stol(pc.error.substr(0, colon))) +
                                 pc.error.substr(colon));
    }
    v0[i] = (int64_t)v.size() / 3;
    t0[i] = (int64_t)vt.size() / 2;
    n0[i] = (int64_t)vn.size() / 3;
    line0[i] = lines;
    tri0[i] = tris;
    v.insert(v.end(), pc.v.begin(), pc.v.end());
    vt.insert(vt.end(), pc.vt.begin(), pc.vt.end());
    vn.insert(vn.end(), pc.vn.begin(), pc.vn.end());
    lines += pc.lines;
    tris += pc.tris;
  }
  out->num_tris = (int)tris;
  out->p.assign(9 * (size_t)tris, 0.f);
  out->n.assign(9 * (size_t)tris, 0.f);
  out->uv.assign(6 * (size_t)tris, 0.f);
  const size_t nv = v.size() / 3, nt = vt.size() / 2, nn = vn.size() / 3;
  std::vector<std::string> errors(npieces);
  for_pieces([&](int i) {
    const obj::Piece& pc = pcs[i];
    int64_t tri = tri0[i];
    // Index as written -> 0-based, -1 when absent; relative indices count back
    // from the vertices read so far (earlier pieces + this one up to the face).
    auto resolve = [](long idx, int64_t before) -> int64_t {
      if (idx > 0) return idx - 1;
      if (idx < 0) return before + idx;
      return -1;
    };
    for (size_t f = 0; f < pc.face_first.size(); ++f) {
      const int first = pc.face_first[f];
      const int last = f + 1 < pc.face_first.size() ? pc.face_first[f + 1] : (int)pc.corners.size();
      const int64_t vb = v0[i] + pc.face_counts[3 * f], tb = t0[i] + pc.face_counts[3 * f + 1],
                    nb = n0[i] + pc.face_counts[3 * f + 2];
      for (int k = first + 1; k + 1 < last; ++k) {
        const int cs[3] = {first, k, k + 1};
        for (int c = 0; c < 3; ++c) {
          const obj::Corner& cr = pc.corners[cs[c]];
          const int64_t iv = resolve(cr.v, vb), it = resolve(cr.t, tb), in = resolve(cr.n, nb);
          if (iv < 0 || (size_t)iv >= nv || in < 0 || (size_t)in >= nn) {
            errors[i] = path + ":" + std::to_string(line0[i] + pc.face_line[f]) +
                        ((iv < 0 || (size_t)iv >= nv) ? ": vertex index out of range"
                                                      : ": face corner without a normal (vn is required)");
            return;
          }
          float* P = &out->p[9 * (size_t)tri + 3 * c];
          float* N = &out->n[9 * (size_t)tri + 3 * c];
          for (int d = 0; d < 3; ++d) {
            P[d] = v[3 * iv + d];
            N[d] = vn[3 * in + d];
          }
          if (it >= 0 && (size_t)it < nt) {
            out->uv[6 * (size_t)tri + 2 * c] = vt[2 * it];
            out->uv[6 * (size_t)tri + 2 * c + 1] = vt[2 * it + 1];
          }
        }
        ++tri;
      }
    }
  });
  for (const std::string& e : errors)
    if (!e.empty()) raise(ORION_ERR_PARSE, e);
}

// meshHandy: inline comma-separated corner data (src/util/strutil.cpp:100-160).
void load_handy(const ParamMap& ps, CornerMesh* out) {
  if (!ps.has("p")) raise(ORION_ERR_PARSE, "meshHandy without p");
  if (!ps.has("n")) raise(ORION_ERR_PARSE, "meshHandy without n (normals are required)");
  auto pv = split_commas(ps.get("p"));
  if (pv.size() % 3 != 0) raise(ORION_ERR_PARSE, "meshHandy p is not a list of points");
  int nv = (int)pv.size() / 3;
  out->num_tris = nv / 3;
  auto nvs = split_commas(ps.get("n"));
  std::vector<std::string> uvs;
  if (ps.has("uv")) uvs = split_commas(ps.get("uv"));
  if (nvs.size() != 3 && nvs.size() < (size_t)nv * 3) raise(ORION_ERR_PARSE, "meshHandy n too short");
  if (!uvs.empty() && uvs.size() < (size_t)nv * 2) raise(ORION_ERR_PARSE, "meshHandy uv too short");
  for (int i = 0; i < out->num_tris * 3; ++i) {
    for (int d = 0; d < 3; ++d) out->p.push_back(parse_float(pv[3 * i + d]));
    for (int d = 0; d < 3; ++d) out->n.push_back(parse_float(nvs.size() == 3 ? nvs[d] : nvs[3 * i + d]));
    for (int d = 0; d < 2; ++d) out->uv.push_back(uvs.empty() ? 0.f : parse_float(uvs[2 * i + d]));
  }
}

// ------------------------------------------------------------ materials

struct TexValue {
  bool present = false;
  bool is_float = false;  // a FloatTexture (usable where the reference casts to one)
  float rgb[3] = {0, 0, 0};
  int32_t image = 0;      // an ImageTexture: the scene's image image - 1
};

// Loads an image file named in the scene and returns its 1-based index in
// the scene's image list (the same file is loaded once).
using ImageLoader = std::function<int32_t(const std::string& name)>;

TexValue texture_of(const XmlNode* mat, const char* tag, const ImageLoader& images) {
  TexValue t;
  const XmlNode* n = mat->child(tag);
  if (!n) return t;
  ParamMap ps = params_of(n);
  std::string type = trim(ps.get("type"));
  if (type == "constant") {
    if (ps.get("color").empty()) return t;
    parse_spectrum(ps.get("color"), t.rgb);
    t.present = true;
  } else if (type == "float") {
    if (ps.get("value").empty()) return t;
    float v = parse_float(ps.get("value"));
    t.rgb[0] = t.rgb[1] = t.rgb[2] = v;
    t.present = t.is_float = true;
  } else if (type == "image") {  // src/util/parser.cpp:438-443
    const std::string fn = trim(ps.get("filename"));
    if (fn.empty()) return t;
    t.image = images(fn);
    t.present = true;
  }
  return t;
}

void need(const TexValue& t, const char* mat, const char* tag) {
  if (!t.present) raise(ORION_ERR_PARSE, std::string(mat) + " material needs <" + tag + ">");
}
void need_float(const TexValue& t, const char* mat, const char* tag) {
  if (!t.present || !t.is_float)
    raise(ORION_ERR_PARSE, std::string(mat) + " material needs a float texture <" + tag + ">");
}
void copy3(float* d, const float* s) { d[0] = s[0], d[1] = s[1], d[2] = s[2]; }
// A Spectrum input: its constant, or the image it is looked up in.
void take(const TexValue& t, float* d, int32_t* tex) {
  copy3(d, t.rgb);
  *tex = t.image;
}

orion_material make_material(const XmlNode* mn, const ImageLoader& images) {
  orion_material m;
  std::memset(&m, 0, sizeof(m));
  std::string type = mn->attr("type") ? mn->attr("type") : "";
  ParamMap mp = params_of(mn);
  if (mp.has("distribution")) {
    std::string d = trim(mp.get("distribution"));
    if (d == "beckmann")
      m.distribution = ORION_DIST_BECKMANN;
    else if (d != "ggx")
      raise(ORION_ERR_UNSUPPORTED, "unknown microfacet distribution '" + d + "'");
  }
  if (type == "matte") {
    TexValue kd = texture_of(mn, "Kd", images), sg = texture_of(mn, "sigma", images);
    need(kd, "matte", "Kd");
    m.type = ORION_MAT_MATTE;
    take(kd, m.Kd, &m.tex[ORION_TEX_KD]);
    if (sg.present && sg.is_float) {
      m.has_sigma = 1;
      m.sigma = sg.rgb[0];
    }
  } else if (type == "mirror") {
    TexValue kr = texture_of(mn, "Kr", images);
    need(kr, "mirror", "Kr");
    m.type = ORION_MAT_MIRROR;
    take(kr, m.Kr, &m.tex[ORION_TEX_KR]);
  } else if (type == "glass") {
    TexValue kr = texture_of(mn, "Kr", images), kt = texture_of(mn, "Kt", images), eta = texture_of(mn, "eta", images),
             rough = texture_of(mn, "roughness", images);
    need(kr, "glass", "Kr");
    need(kt, "glass", "Kt");
    need_float(eta, "glass", "eta");
    need_float(rough, "glass", "roughness");
    m.type = ORION_MAT_GLASS;
    take(kr, m.Kr, &m.tex[ORION_TEX_KR]);
    take(kt, m.Kt, &m.tex[ORION_TEX_KT]);
    m.eta = eta.rgb[0];
    m.roughness = rough.rgb[0];
  } else if (type == "plastic") {
    TexValue kd = texture_of(mn, "Kd", images), ks = texture_of(mn, "Ks", images), rough = texture_of(mn, "roughness", images);
    need(kd, "plastic", "Kd");
    need(ks, "plastic", "Ks");
    need_float(rough, "plastic", "roughness");
    m.type = ORION_MAT_PLASTIC;
    take(kd, m.Kd, &m.tex[ORION_TEX_KD]);
    take(ks, m.Ks, &m.tex[ORION_TEX_KS]);
    m.roughness = rough.rgb[0];
  } else if (type == "metal") {
    const XmlNode* en = mn->child("eta");
    const XmlNode* kn = mn->child("k");
    if ((en && params_of(en).has("SPD")) || (kn && params_of(kn).has("SPD")))
      raise(ORION_ERR_UNSUPPORTED, "metal SPD files are not supported");
    TexValue eta = texture_of(mn, "eta", images), k = texture_of(mn, "k", images), rough = texture_of(mn, "roughness", images);
    m.type = ORION_MAT_METAL;
    // src/material/metal.cpp:98-140: explicit eta, k and roughness are used
    // only when all three are given; otherwise the named-metal branch runs,
    // which leaves eta = k = 0 unless a metalName is set.
    if (eta.present && k.present && rough.present && rough.is_float) {
      take(eta, m.eta_rgb, &m.tex[ORION_TEX_ETA]);
      take(k, m.k, &m.tex[ORION_TEX_K]);
      m.roughness = rough.rgb[0];
    } else {
      if (mp.has("metalName")) raise(ORION_ERR_UNSUPPORTED, "named metals are not supported");
      m.roughness = (rough.present && rough.is_float) ? rough.rgb[0] : 0.1f;
    }
  } else if (type == "uber") {
    const char* tags[5] = {"Kd", "Ks", "Kr", "Kt", "opacity"};
    float* dst[5] = {m.Kd, m.Ks, m.Kr, m.Kt, m.opacity};
    const int slot[5] = {ORION_TEX_KD, ORION_TEX_KS, ORION_TEX_KR, ORION_TEX_KT, ORION_TEX_OPACITY};
    for (int i = 0; i < 5; ++i) {
      TexValue t = texture_of(mn, tags[i], images);
      need(t, "uber", tags[i]);
      take(t, dst[i], &m.tex[slot[i]]);
    }
    TexValue rough = texture_of(mn, "roughness", images), eta = texture_of(mn, "eta", images);
    need_float(rough, "uber", "roughness");
    need_float(eta, "uber", "eta");
    m.type = ORION_MAT_UBER;
    m.roughness = rough.rgb[0];
    m.eta = eta.rgb[0];
  } else if (type == "kdsubsurface") {
    raise(ORION_ERR_UNSUPPORTED, "kdsubsurface material is not supported");
  } else {
    raise(ORION_ERR_PARSE, "material without a known type: '" + type + "'");
  }
  return m;
}

// ---------------------------------------------------------------- loader

void set_rows(float out[12], const Mat4& a) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) out[4 * r + c] = a.m[r][c];
}

class Loader {
 public:
  Loader(const std::string& path, HostScene* out) : path_(path), out_(out), reuse_(8) {}

  void run() {
    std::string text;
    if (!read_file(path_, &text)) raise(ORION_ERR_IO, "cannot read scene " + path_);
    std::string err;
    XmlReader reader(text);
    root_ = reader.parse_document(&err);
    if (!root_) raise(ORION_ERR_PARSE, path_ + ": " + err);
    size_t slash = path_.find_last_of('/');
    scene_dir_ = slash == std::string::npos ? std::string() : path_.substr(0, slash + 1);
    const XmlNode* res = root_->child("Resource");
    if (!res || !res->attr("filename")) raise(ORION_ERR_PARSE, "missing <Resource filename=...>");
    std::string rp = res->attr("filename");
    res_dir_ = (!rp.empty() && rp[0] == '/') ? rp : scene_dir_ + rp;
    camera();
    models();
    lights();
    sampler();
    integrator();
    envmaps();
    out_->source = path_;
  }

 private:
  std::string path_, scene_dir_, res_dir_;
  HostScene* out_;
  std::unique_ptr<XmlNode> root_;
  std::vector<Xform> reuse_;
  std::map<std::string, int> named_;
  std::map<std::string, int32_t> image_index_;

  Xform transform_of(const XmlNode* n) {
    const XmlNode* t = n->child("Transform");
    return t ? make_transform(t, &reuse_) : Xform();
  }

  void camera() {
    const XmlNode* c = root_->child("Camera");
    if (!c) raise(ORION_ERR_PARSE, "no <Camera>");
    std::string type = trim(c->attr("type") ? c->attr("type") : "");
    if (type != "pinhole") raise(ORION_ERR_UNSUPPORTED, "camera type '" + type + "'");
    ParamMap ps = params_of(c);
    Xform t = transform_of(c);
    orion_camera& cam = out_->camera;
    std::memcpy(cam.c2w, t.m.m, sizeof(cam.c2w));
    auto fs = split_commas(ps.get("filmsize"));
    if (fs.size() < 2) raise(ORION_ERR_PARSE, "camera needs filmsize=\"W,H\"");
    cam.width = std::atoi(fs[0].c_str());
    cam.height = std::atoi(fs[1].c_str());
    if (cam.width <= 0 || cam.height <= 0) raise(ORION_ERR_PARSE, "film size must be positive");
    if (!ps.has("fov")) raise(ORION_ERR_PARSE, "camera needs fov");
    cam.fov = parse_float(ps.get("fov"));
    cam.lens_radius = 0.f;
    cam.focal_distance = 0.f;
    if (ps.has("lensRadius")) {
      cam.lens_radius = parse_float(ps.get("lensRadius"));
      cam.focal_distance = parse_float(ps.get("focalDistance"));
    }
  }

  int material_index(const XmlNode* mn) {
    if (!mn) raise(ORION_ERR_PARSE, "<Model> without <Material>");
    const char* named = mn->attr("named");
    if (named && *named) {
      auto it = named_.find(named);
      if (it == named_.end()) raise(ORION_ERR_PARSE, std::string("no material named '") + named + "'");
      return it->second;
    }
    out_->materials.push_back(make_material(mn, [this](const std::string& fn) { return texture_image(fn); }));
    int idx = (int)out_->materials.size() - 1;
    const char* name = mn->attr("name");
    if (name && *name) named_.insert(std::make_pair(std::string(name), idx));
    return idx;
  }

  void models() {
    for (const XmlNode* model : root_->all("Model")) {
      Xform t = transform_of(model);
      std::string type = model->attr("type") ? model->attr("type") : "";
      CornerMesh mesh;
      if (type == "mesh") {
        const char* fn = model->attr("filename");
        if (!fn) raise(ORION_ERR_PARSE, "mesh <Model> without filename");
        load_obj(res_dir_ + fn, &mesh);
      } else if (type == "meshHandy") {
        load_handy(params_of(model), &mesh);
      } else {
        raise(ORION_ERR_PARSE, "unknown model type '" + type + "'");
      }
      int mat = material_index(model->child("Material"));
      const XmlNode* al = model->child("AreaLight");
      float le[3] = {0, 0, 0};
      if (al) {
        ParamMap ap = params_of(al);
        if (!ap.has("Le")) raise(ORION_ERR_PARSE, "<AreaLight> without Le");
        parse_spectrum(ap.get("Le"), le);
      }
      // createTriangleMesh (src/core/triangle.cpp:137-151): bake the model
      // transform into corner positions and (un-normalised) normals, in
      // parallel slices of the mesh (each corner's result is independent).
      const size_t base = out_->positions.size();
      out_->positions.resize(base + 9 * (size_t)mesh.num_tris);
      out_->normals.resize(base + 9 * (size_t)mesh.num_tris);
      out_->uvs.insert(out_->uvs.end(), mesh.uv.begin(), mesh.uv.begin() + 6 * (size_t)mesh.num_tris);
      {
        const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
        const int parts = mesh.num_tris < 65536 ? 1 : hw;
        std::vector<std::thread> th;
        for (int pt = 0; pt < parts; ++pt)
          th.emplace_back([&, pt] {
            const int64_t b = (int64_t)mesh.num_tris * pt / parts, e = (int64_t)mesh.num_tris * (pt + 1) / parts;
            for (int64_t c = 3 * b; c < 3 * e; ++c) {
              t.point(&mesh.p[3 * c], &out_->positions[base + 3 * c]);
              t.normal(&mesh.n[3 * c], &out_->normals[base + 3 * c]);
            }
          });
        for (auto& x : th) x.join();
      }
      for (int tri = 0; tri < mesh.num_tris; ++tri) {
        int32_t prim = (int32_t)out_->material_of_prim.size();
        out_->material_of_prim.push_back(mat);
        if (al) {
          orion_light l;
          std::memset(&l, 0, sizeof(l));
          l.type = ORION_LIGHT_AREA;
          l.prim = prim;
          copy3(l.L, le);
          out_->lights.push_back(l);
          out_->light_of_prim.push_back((int32_t)out_->lights.size() - 1);
        } else {
          out_->light_of_prim.push_back(-1);
        }
      }
    }
  }

  void lights() {
    for (const XmlNode* ln : root_->all("Light")) {
      std::string type = trim(ln->attr("type") ? ln->attr("type") : "");
      ParamMap ps = params_of(ln);
      orion_light l;
      std::memset(&l, 0, sizeof(l));
      if (type == "point") {
        // src/light/point.cpp:35-41
        l.type = ORION_LIGHT_POINT;
        parse_spectrum(ps.get("I"), l.L);
        float from[3], zero[3] = {0, 0, 0};
        parse_vec3(ps.get("from"), from, "point light from");
        Xform::translate(from[0], from[1], from[2]).point(zero, l.p);
      } else if (type == "spot") {
        // src/light/spot.cpp:46-58 with spot.h:22-25 (falloff start taken
        // from the falloffStart argument)
        l.type = ORION_LIGHT_SPOT;
        parse_spectrum(ps.get("intensity"), l.L);
        float cone = parse_float(ps.get("angle"));
        float delta = parse_float(ps.get("delta"));
        float from[3], to[3], zero[3] = {0, 0, 0};
        parse_vec3(ps.get("from"), from, "spot from");
        parse_vec3(ps.get("to"), to, "spot to");
        float d0[3] = {to[0] - from[0], to[1] - from[1], to[2] - from[2]}, dir[3], x[3], y[3];
        v_normalize(d0, dir);
        if (std::fabs(dir[0]) > std::fabs(dir[1])) {
          float inv = 1.f / std::sqrt(dir[0] * dir[0] + dir[2] * dir[2]);
          y[0] = -dir[2] * inv;
          y[1] = 0 * inv;
          y[2] = dir[0] * inv;
        } else {
          float inv = 1.f / std::sqrt(dir[1] * dir[1] + dir[2] * dir[2]);
          y[0] = 0 * inv;
          y[1] = dir[2] * inv;
          y[2] = -dir[1] * inv;
        }
        v_cross(y, dir, x);
        Xform dir_to_z(Mat4::make(x[0], x[1], x[2], 0, y[0], y[1], y[2], 0, dir[0], dir[1], dir[2], 0, 0, 0, 0, 1));
        Xform l2w = Xform::translate(from[0], from[1], from[2]) * dir_to_z.inverse();
        l2w.point(zero, l.p);
        set_rows(l.l2w, l2w.m);
        set_rows(l.w2l, l2w.minv);
        l.cos_total = std::cos(radians_f(cone));
        l.cos_falloff = std::cos(radians_f(cone - delta));
      } else if (type == "distant") {
        // src/light/distant.cpp:49-56 and distant.h:25
        l.type = ORION_LIGHT_DISTANT;
        parse_spectrum(ps.get("L"), l.L);
        float from[3], to[3];
        parse_vec3(ps.get("from"), from, "distant from");
        parse_vec3(ps.get("to"), to, "distant to");
        float d0[3] = {to[0] - from[0], to[1] - from[1], to[2] - from[2]}, dir[3], dw[3];
        v_normalize(d0, dir);
        Xform::translate(from[0], from[1], from[2]).vector(dir, dw);
        v_normalize(dw, l.dir);
      } else {
        continue;  // the reference ignores unknown light types
      }
      out_->lights.push_back(l);
    }
  }

  void sampler() {
    const XmlNode* s = root_->child("Sampler");
    if (!s) raise(ORION_ERR_PARSE, "no <Sampler>");
    std::string type = s->attr("type") ? s->attr("type") : "";
    if (type != "sobol") raise(ORION_ERR_UNSUPPORTED, "sampler '" + type + "' (only sobol)");
  }

  void integrator() {
    const XmlNode* n = root_->child("Integrator");
    if (!n) raise(ORION_ERR_PARSE, "no <Integrator>");
    std::string type = trim(n->attr("type") ? n->attr("type") : "");
    ParamMap ps = params_of(n);
    if (type == "sppm") {  // createSPPMIntegrator (src/integrator/sppm.cpp:324-333)
      for (const char* k : {"numIterations", "maxDepth", "photonsPerIteration", "initRadius"})
        if (!ps.has(k)) raise(ORION_ERR_PARSE, std::string("sppm integrator needs ") + k);
      out_->integrator = ORION_INTEGRATOR_SPPM;
      out_->sppm.iterations = parse_int(ps.get("numIterations"));
      out_->sppm.max_depth = parse_int(ps.get("maxDepth"));
      out_->sppm.photons_per_iter = parse_int(ps.get("photonsPerIteration"));
      out_->sppm.initial_radius = parse_float(ps.get("initRadius"));
      out_->max_depth = out_->sppm.max_depth;
      out_->spp = out_->sppm.iterations;
      return;
    }
    if (type != "path") raise(ORION_ERR_UNSUPPORTED, "integrator '" + type + "' (path or sppm)");
    if (!ps.has("maxDepth") || !ps.has("nSamplesPerPixel"))
      raise(ORION_ERR_PARSE, "path integrator needs maxDepth and nSamplesPerPixel");
    out_->integrator = ORION_INTEGRATOR_PATH;
    out_->max_depth = parse_int(ps.get("maxDepth"));
    out_->spp = parse_int(ps.get("nSamplesPerPixel"));
  }

  // loadImage (src/texture/imagetexture.cpp:28-52): 8-bit texels times
  // 1/255; returns the image's 1-based index in the scene (a file is loaded once).
  int32_t load_image(const std::string& file) {
    auto it = image_index_.find(file);
    if (it != image_index_.end()) return it->second;
    Image8 im8;
    std::string ierr;
    if (!load_image8(file, &im8, &ierr)) raise(ORION_ERR_IO, ierr);
    if (im8.channels != 3 && im8.channels != 4)
      raise(ORION_ERR_UNSUPPORTED, file + ": only 3- or 4-channel images are read by the reference");
    HostImage hi;
    hi.width = im8.width;
    hi.height = im8.height;
    hi.rgb.resize(im8.rgb.size());
    const float inv255 = 0.0039215686274509803921568627451f;  // color_CharToFloat
    for (size_t i = 0; i < im8.rgb.size(); ++i) hi.rgb[i] = im8.rgb[i] * inv255;
    out_->images.push_back(std::move(hi));
    const int32_t idx = (int32_t)out_->images.size();
    image_index_[file] = idx;
    return idx;
  }

  // An image texture's file: absolute, or found in the resource directory,
  // the scene's directory or the working directory, in that order.
  int32_t texture_image(const std::string& name) {
    if (name[0] == '/') return load_image(name);
    for (const std::string& dir : {res_dir_, scene_dir_}) {
      std::FILE* f = std::fopen((dir + name).c_str(), "rb");
      if (f) {
        std::fclose(f);
        return load_image(dir + name);
      }
    }
    return load_image(name);
  }

  void envmaps() {
    // src/light/envmap.cpp:116-135
    for (const XmlNode* en : root_->all("Envmap")) {
      Xform transform = transform_of(en);
      ParamMap ps = params_of(en);
      orion_light l;
      std::memset(&l, 0, sizeof(l));
      l.type = ORION_LIGHT_ENV;
      if (ps.has("name")) {
        // Envmap(...) reads the image from the resource directory
        // (src/light/envmap.cpp:120, :14-22).
        l.image = load_image(res_dir_ + trim(ps.get("name")));
      }
      if (ps.has("L"))
        parse_spectrum(ps.get("L"), l.L);
      else
        l.L[0] = l.L[1] = l.L[2] = 1.f;
      if (!ps.has("worldUp")) raise(ORION_ERR_PARSE, "<Envmap> needs worldUp");
      float up0[3], up[3];
      parse_vec3(ps.get("worldUp"), up0, "worldUp");
      v_normalize(up0, up);
      const float env_up[3] = {0, 0, 1};
      float c = v_dot(up, env_up);
      Xform t;
      if (c < 0.99 && c > -0.99) {
        // The reference calls the C library's double acos here
        // (src/light/envmap.cpp:126, unqualified acos on a float).
        float angle = (float)::acos((double)v_dot(up, env_up));
        float axis[3];
        v_cross(env_up, up, axis);
        t = Xform::rotate(degrees_f(angle), axis);
      }
      Xform l2w = t * transform;
      set_rows(l.l2w, l2w.m);
      set_rows(l.w2l, l2w.minv);
      out_->lights.push_back(l);
    }
  }
};

}  // namespace

void HostScene::desc(orion_scene_desc* d) const {
  std::memset(d, 0, sizeof(*d));
  d->num_prims = num_prims();
  d->positions = positions.data();
  d->normals = normals.data();
  d->uvs = uvs.empty() ? nullptr : uvs.data();
  d->material_of_prim = material_of_prim.data();
  d->light_of_prim = light_of_prim.data();
  d->num_materials = (int32_t)materials.size();
  d->num_lights = (int32_t)lights.size();
  d->materials = materials.data();
  d->lights = lights.data();
  d->camera = camera;
  d->spp = spp;
  d->max_depth = max_depth;
  d->num_images = (int32_t)image_desc.size();
  d->images = image_desc.empty() ? nullptr : image_desc.data();
  d->integrator = integrator;
  d->sppm = sppm;
}

void HostScene::index_images() {
  image_desc.clear();
  for (const HostImage& im : images) image_desc.push_back(orion_image{im.width, im.height, im.rgb.data()});
}

int load_ori(const std::string& path, HostScene* out, std::string* err) {
  try {
    Loader(path, out).run();
    out->index_images();
  } catch (const LoadError& e) {
    *err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    *err = "out of host memory while loading " + path;
    return ORION_ERR_NOMEM;
  }
  return ORION_OK;
}

int scene_from_desc(const orion_scene_desc& d, HostScene* out, std::string* err) {
  if (d.num_prims < 0 || (d.num_prims > 0 && (!d.positions || !d.normals || !d.material_of_prim))) {
    *err = "scene description: missing primitive arrays";
    return ORION_ERR_INVALID;
  }
  if (d.num_materials <= 0 || !d.materials) {
    *err = "scene description: no materials";
    return ORION_ERR_INVALID;
  }
  if (d.num_lights < 0 || (d.num_lights > 0 && !d.lights)) {
    *err = "scene description: bad light array";
    return ORION_ERR_INVALID;
  }
  if (d.camera.width <= 0 || d.camera.height <= 0) {
    *err = "scene description: film size must be positive";
    return ORION_ERR_INVALID;
  }
  size_t T = (size_t)d.num_prims;
  out->positions.assign(d.positions, d.positions + 9 * T);
  out->normals.assign(d.normals, d.normals + 9 * T);
  if (d.uvs)
    out->uvs.assign(d.uvs, d.uvs + 6 * T);
  else
    out->uvs.assign(6 * T, 0.f);
  out->material_of_prim.assign(d.material_of_prim, d.material_of_prim + T);
  if (d.light_of_prim)
    out->light_of_prim.assign(d.light_of_prim, d.light_of_prim + T);
  else
    out->light_of_prim.assign(T, -1);
  out->materials.assign(d.materials, d.materials + d.num_materials);
  out->lights.assign(d.lights, d.lights + d.num_lights);
  if (d.num_images < 0 || (d.num_images > 0 && !d.images)) {
    *err = "scene description: bad image array";
    return ORION_ERR_INVALID;
  }
  out->images.clear();
  for (int i = 0; i < d.num_images; ++i) {
    const orion_image& im = d.images[i];
    if (im.width <= 0 || im.height <= 0 || !im.rgb || (int64_t)im.width * im.height > (1LL << 28)) {
      *err = "scene description: bad image " + std::to_string(i);
      return ORION_ERR_INVALID;
    }
    HostImage hi;
    hi.width = im.width;
    hi.height = im.height;
    hi.rgb.assign(im.rgb, im.rgb + 3 * (size_t)im.width * im.height);
    out->images.push_back(std::move(hi));
  }
  out->index_images();
  for (const orion_light& l : out->lights)
    if (l.image < 0 || l.image > d.num_images || (l.image > 0 && l.type != ORION_LIGHT_ENV)) {
      *err = "scene description: light image index out of range";
      return ORION_ERR_INVALID;
    }
  for (size_t i = 0; i < T; ++i) {
    if (out->material_of_prim[i] < 0 || out->material_of_prim[i] >= d.num_materials) {
      *err = "scene description: material index out of range at primitive " + std::to_string(i);
      return ORION_ERR_INVALID;
    }
    int32_t li = out->light_of_prim[i];
    if (li < -1 || li >= d.num_lights || (li >= 0 && (d.lights[li].type != ORION_LIGHT_AREA || d.lights[li].prim != (int32_t)i))) {
      *err = "scene description: light_of_prim inconsistent at primitive " + std::to_string(i);
      return ORION_ERR_INVALID;
    }
  }
  for (int i = 0; i < d.num_lights; ++i) {
    const orion_light& l = d.lights[i];
    if (l.type < ORION_LIGHT_AREA || l.type > ORION_LIGHT_ENV || (l.type == ORION_LIGHT_AREA && (l.prim < 0 || l.prim >= d.num_prims))) {
      *err = "scene description: bad light " + std::to_string(i);
      return ORION_ERR_INVALID;
    }
  }
  for (int i = 0; i < d.num_materials; ++i)
    if (d.materials[i].type < ORION_MAT_MATTE || d.materials[i].type > ORION_MAT_UBER) {
      *err = "scene description: bad material type at " + std::to_string(i);
      return ORION_ERR_INVALID;
    }
  if (d.integrator != ORION_INTEGRATOR_PATH && d.integrator != ORION_INTEGRATOR_SPPM) {
    *err = "scene description: unknown integrator";
    return ORION_ERR_INVALID;
  }
  out->camera = d.camera;
  out->spp = d.spp;
  out->max_depth = d.max_depth;
  out->integrator = d.integrator;
  out->sppm = d.sppm;
  out->source.clear();
  return ORION_OK;
}

}  // namespace orion_gb300
