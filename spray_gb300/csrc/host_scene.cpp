// Host-side scene I/O and the wavelet generator.  See host_scene.h.
#include "host_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace sg {

// ---------------------------------------------------------------- transforms
// The column-major 4x4 helpers below evaluate products in the order of glm's
// translate/scale/rotate and mat4 * vec4, which SpRay builds and applies its
// domain matrices with (src/io/scene_loader.cc:149-186, 351-357;
// src/render/trimesh_buffer.cc:141-153), so a translate-only matrix moves a
// vertex by exactly one float add per coordinate.  Like SpRay
// (src/render/scene.inl:151), an identity matrix is not applied.

Mat4 Mat4::identity() {
  Mat4 r;
  for (int c = 0; c < 4; ++c)
    for (int k = 0; k < 4; ++k) r.m[c][k] = (c == k) ? 1.f : 0.f;
  return r;
}

bool Mat4::isIdentity() const {
  Mat4 id = identity();
  for (int c = 0; c < 4; ++c)
    for (int k = 0; k < 4; ++k)
      if (m[c][k] != id.m[c][k]) return false;
  return true;
}

static void colMulAdd(float out[4], const float a[4], float s) {
  for (int k = 0; k < 4; ++k) out[k] = a[k] * s;
}

Mat4 translate(const Mat4& m, float x, float y, float z) {
  Mat4 r = m;
  for (int k = 0; k < 4; ++k) {
    float v = m.m[0][k] * x;
    v = v + m.m[1][k] * y;
    v = v + m.m[2][k] * z;
    v = v + m.m[3][k];
    r.m[3][k] = v;
  }
  return r;
}

Mat4 scale(const Mat4& m, float x, float y, float z) {
  Mat4 r = m;
  colMulAdd(r.m[0], m.m[0], x);
  colMulAdd(r.m[1], m.m[1], y);
  colMulAdd(r.m[2], m.m[2], z);
  return r;
}

Mat4 rotate(const Mat4& m, float a, int axis_id) {
  float axis[3] = {0, 0, 0};
  axis[axis_id] = 1.f;
  const float c = std::cos(a);
  const float s = std::sin(a);
  float temp[3];
  for (int i = 0; i < 3; ++i) temp[i] = (1.f - c) * axis[i];
  float R[3][3];
  R[0][0] = c + temp[0] * axis[0];
  R[0][1] = temp[0] * axis[1] + s * axis[2];
  R[0][2] = temp[0] * axis[2] - s * axis[1];
  R[1][0] = temp[1] * axis[0] - s * axis[2];
  R[1][1] = c + temp[1] * axis[1];
  R[1][2] = temp[1] * axis[2] + s * axis[0];
  R[2][0] = temp[2] * axis[0] + s * axis[1];
  R[2][1] = temp[2] * axis[1] - s * axis[0];
  R[2][2] = c + temp[2] * axis[2];
  Mat4 r = m;
  for (int col = 0; col < 3; ++col) {
    for (int k = 0; k < 4; ++k) {
      float v = m.m[0][k] * R[col][0];
      v = v + m.m[1][k] * R[col][1];
      v = v + m.m[2][k] * R[col][2];
      r.m[col][k] = v;
    }
  }
  return r;
}

// m * vec4(in, 1) as glm evaluates mat4 * vec4 (type_mat4x4.inl, since glm
// 0.9.5): the pairwise sum (m[0]*x + m[1]*y) + (m[2]*z + m[3]*w).  SpRay
// transforms domain vertices (src/render/trimesh_buffer.cc:141-153) and the
// object-bound corners (src/io/scene_loader.cc:351-357) with it.
void transformPoint(const Mat4& m, const float in[3], float out[3]) {
  for (int k = 0; k < 3; ++k) {
    const float add0 = m.m[0][k] * in[0] + m.m[1][k] * in[1];
    const float add1 = m.m[2][k] * in[2] + m.m[3][k] * 1.0f;
    out[k] = add0 + add1;
  }
}

// ---------------------------------------------------------------- .spray
static std::runtime_error parseError(const std::string& file, int line,
                                     const std::string& what) {
  std::ostringstream os;
  os << file << ":" << line << ": " << what;
  return std::runtime_error(os.str());
}

static float tokf(const std::vector<std::string>& t, size_t i) {
  return (float)std::atof(t[i].c_str());
}

SceneDesc loadSceneFile(const std::string& filename, const std::string& ply_path) {
  std::ifstream in(filename);
  if (!in.is_open()) throw std::runtime_error("unable to open scene file " + filename);
  SceneDesc sd;
  std::string line;
  int lineno = 0;
  auto cur = [&](int ln) -> Domain& {
    if (sd.domains.empty()) throw parseError(filename, ln, "domain attribute before 'domain'");
    return sd.domains.back();
  };
  while (std::getline(in, line)) {
    ++lineno;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::vector<std::string> t;
    {
      // tokens are separated by single spaces exactly like strtok(" ")
      std::string copy(line);
      for (char* tok = std::strtok(&copy[0], " "); tok; tok = std::strtok(nullptr, " ")) t.emplace_back(tok);
    }
    if (t.empty()) continue;
    const std::string& tag = t[0];
    if (tag[0] == '#') continue;
    if (tag == "domain") {
      Domain d;
      d.id = (int)sd.domains.size();
      sd.domains.push_back(d);
    } else if (tag == "file") {
      if (t.size() != 2) throw parseError(filename, lineno, "file expects 1 argument");
      cur(lineno).filename = ply_path.empty() ? t[1] : ply_path + "/" + t[1];
    } else if (tag == "mtl") {
      Domain& d = cur(lineno);
      if (t.size() < 2) throw parseError(filename, lineno, "mtl expects a type");
      if (t[1] == "diffuse" || t[1] == "mirror") {
        if (t.size() != 5) throw parseError(filename, lineno, "mtl " + t[1] + " expects r g b");
        d.bsdf_type = (t[1] == "diffuse") ? BSDF_DIFFUSE : BSDF_MIRROR;
        for (int i = 0; i < 3; ++i) d.bsdf_params[i] = tokf(t, 2 + i);
      } else if (t[1] == "glass" || t[1] == "transmission") {
        if (t.size() != 4) throw parseError(filename, lineno, "mtl " + t[1] + " expects etaA etaB");
        d.bsdf_type = (t[1] == "glass") ? BSDF_GLASS : BSDF_TRANSMISSION;
        d.bsdf_params[0] = tokf(t, 2);
        d.bsdf_params[1] = tokf(t, 3);
        d.bsdf_params[2] = 0.f;
      } else {
        throw parseError(filename, lineno, "unknown material type " + t[1]);
      }
    } else if (tag == "bound") {
      if (t.size() != 7) throw parseError(filename, lineno, "bound expects 6 numbers");
      Domain& d = cur(lineno);
      for (int i = 0; i < 6; ++i) d.object_bounds[i] = tokf(t, 1 + i);
    } else if (tag == "scale") {
      if (t.size() != 4) throw parseError(filename, lineno, "scale expects 3 numbers");
      Domain& d = cur(lineno);
      d.transform = scale(d.transform, tokf(t, 1), tokf(t, 2), tokf(t, 3));
    } else if (tag == "rotate") {
      if (t.size() != 3) throw parseError(filename, lineno, "rotate expects axis and degrees");
      int axis = t[1] == "x" ? 0 : t[1] == "y" ? 1 : t[1] == "z" ? 2 : -1;
      if (axis < 0) throw parseError(filename, lineno, "invalid axis name " + t[1]);
      double deg = std::atof(t[2].c_str());
      float rad = (float)(deg * 0.01745329251994329576923690768489);
      Domain& d = cur(lineno);
      d.transform = rotate(d.transform, rad, axis);
    } else if (tag == "translate") {
      if (t.size() != 4) throw parseError(filename, lineno, "translate expects 3 numbers");
      Domain& d = cur(lineno);
      d.transform = translate(d.transform, tokf(t, 1), tokf(t, 2), tokf(t, 3));
    } else if (tag == "face") {
      if (t.size() != 2) throw parseError(filename, lineno, "face expects a count");
      cur(lineno).num_faces = std::stoull(t[1]);
    } else if (tag == "vertex") {
      if (t.size() != 2) throw parseError(filename, lineno, "vertex expects a count");
      cur(lineno).num_vertices = std::stoull(t[1]);
    } else if (tag == "light") {
      if (t.size() < 2) throw parseError(filename, lineno, "light expects a type");
      Light l;
      if (t[1] == "point") {
        if (t.size() != 8) throw parseError(filename, lineno, "light point expects 6 numbers");
        l.type = LIGHT_POINT;
        for (int i = 0; i < 3; ++i) l.position[i] = tokf(t, 2 + i);
        for (int i = 0; i < 3; ++i) l.radiance[i] = tokf(t, 5 + i);
      } else if (t[1] == "diffuse") {
        if (t.size() != 5) throw parseError(filename, lineno, "light diffuse expects 3 numbers");
        l.type = LIGHT_DIFFUSE;
        for (int i = 0; i < 3; ++i) l.radiance[i] = tokf(t, 2 + i);
      } else if (t[1] == "quad") {
        // extension: light quad p0(3) edge1(3) edge2(3) radiance(3)
        if (t.size() != 14) throw parseError(filename, lineno, "light quad expects 12 numbers");
        l.type = LIGHT_QUAD;
        for (int i = 0; i < 3; ++i) l.position[i] = tokf(t, 2 + i);
        for (int i = 0; i < 3; ++i) l.edge1[i] = tokf(t, 5 + i);
        for (int i = 0; i < 3; ++i) l.edge2[i] = tokf(t, 8 + i);
        for (int i = 0; i < 3; ++i) l.radiance[i] = tokf(t, 11 + i);
      } else {
        throw parseError(filename, lineno, "unknown light source " + t[1]);
      }
      sd.lights.push_back(l);
    } else {
      throw parseError(filename, lineno, "unknown tag name " + tag);
    }
  }
  if (sd.domains.empty()) throw std::runtime_error("no domains in scene file " + filename);
  for (auto& d : sd.domains) {
    const float* b = d.object_bounds;
    float mn[3] = {b[0], b[1], b[2]}, mx[3] = {b[3], b[4], b[5]};
    transformPoint(d.transform, mn, d.world_bounds);
    transformPoint(d.transform, mx, d.world_bounds + 3);
  }
  return sd;
}

// ---------------------------------------------------------------- PLY
namespace {
enum { T_UNDEF = -1, T_CHAR, T_UCHAR, T_SHORT, T_USHORT, T_INT, T_UINT, T_FLOAT, T_DOUBLE };
int plyType(const std::string& s) {
  if (s == "char" || s == "int8") return T_CHAR;
  if (s == "uchar" || s == "uint8") return T_UCHAR;
  if (s == "short" || s == "int16") return T_SHORT;
  if (s == "ushort" || s == "uint16") return T_USHORT;
  if (s == "int" || s == "int32") return T_INT;
  if (s == "uint" || s == "uint32") return T_UINT;
  if (s == "float" || s == "float32") return T_FLOAT;
  if (s == "double" || s == "float64") return T_DOUBLE;
  throw std::runtime_error("ply: unknown data type " + s);
}
int plySize(int t) {
  switch (t) {
    case T_CHAR: case T_UCHAR: return 1;
    case T_SHORT: case T_USHORT: return 2;
    case T_INT: case T_UINT: case T_FLOAT: return 4;
    case T_DOUBLE: return 8;
  }
  throw std::runtime_error("ply: bad type");
}
uint32_t readUIntLE(std::istream& in, int bytes) {
  unsigned char b[8] = {0};
  in.read((char*)b, bytes);
  uint32_t v = 0;
  for (int i = bytes - 1; i >= 0; --i) v = (v << 8) | b[i];
  if (bytes > 4) v = (uint32_t)(b[0] | (b[1] << 8) | (b[2] << 16) | ((uint32_t)b[3] << 24));
  return v;
}
}  // namespace

void readPly(const std::string& filename, Mesh* mesh) {
  std::ifstream f(filename, std::ios::in | std::ios::binary);
  if (!f.is_open()) throw std::runtime_error("unable to open ply file " + filename);
  std::string line;
  std::getline(f, line);
  if (!line.empty() && line.back() == '\r') line.pop_back();
  if (line != "ply") throw std::runtime_error(filename + ": unknown file type");
  int format = -1;  // 0 ascii, 1 binary little endian
  uint64_t nv = 0, nf = 0;
  int elem = -1;  // 0 vertex, 1 face
  int order[2] = {-1, -1};
  int nelem = 0;
  int vtype = T_UNDEF, ltype = T_UNDEF, itype = T_UNDEF;
  bool has_color = false;
  int ncolor = 0, npos = 0;
  bool end_header = false;
  while (std::getline(f, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::istringstream ss(line);
    std::string w;
    ss >> w;
    if (w == "format") {
      ss >> w;
      if (w == "ascii") format = 0;
      else if (w == "binary_little_endian") format = 1;
      else throw std::runtime_error(filename + ": unsupported ply format " + w);
    } else if (w == "element") {
      std::string name;
      uint64_t n = 0;
      ss >> name >> n;
      if (nelem >= 2) throw std::runtime_error(filename + ": more than two ply elements");
      if (name == "vertex") { elem = 0; nv = n; }
      else if (name == "face") { elem = 1; nf = n; }
      else throw std::runtime_error(filename + ": unknown element " + name);
      order[nelem++] = elem;
    } else if (w == "property") {
      if (elem == 0) {
        std::string dt, name;
        ss >> dt >> name;
        if (name == "x" || name == "y" || name == "z") {
          int t = plyType(dt);
          if (t != T_FLOAT) throw std::runtime_error(filename + ": vertex coordinates must be float");
          vtype = t;
          ++npos;
        } else if (name == "red" || name == "green" || name == "blue") {
          int t = plyType(dt);
          if (t != T_UCHAR) throw std::runtime_error(filename + ": colors must be uchar");
          ++ncolor;
          has_color = true;
        } else {
          throw std::runtime_error(filename + ": unknown property " + name);
        }
      } else if (elem == 1) {
        std::string list, lt, it, name;
        ss >> list >> lt >> it >> name;
        if (list != "list") throw std::runtime_error(filename + ": face property must be a list");
        ltype = plyType(lt);
        itype = plyType(it);
        if (name != "vertex_index" && name != "vertex_indices")
          throw std::runtime_error(filename + ": unknown property " + name);
      }
    } else if (w == "end_header") {
      end_header = true;
      break;
    }
  }
  if (!end_header || format < 0 || nv == 0 || nf == 0 || npos != 3 || vtype != T_FLOAT)
    throw std::runtime_error(filename + ": malformed ply header");
  if (has_color && ncolor != 3) throw std::runtime_error(filename + ": partial colors");
  mesh->vertices.assign(3 * nv, 0.f);
  mesh->faces.assign(3 * nf, 0u);
  mesh->colors.assign(nv, 0u);
  mesh->has_color = has_color;
  for (int e = 0; e < nelem; ++e) {
    if (order[e] == 0) {
      for (uint64_t n = 0; n < nv; ++n) {
        if (format == 1) {
          float xyz[3];
          f.read((char*)xyz, 12);
          for (int i = 0; i < 3; ++i) mesh->vertices[3 * n + i] = xyz[i];
          if (has_color) {
            unsigned char c[3];
            f.read((char*)c, 3);
            mesh->colors[n] = ((uint32_t)c[0] << 16) | ((uint32_t)c[1] << 8) | c[2];
          }
        } else {
          if (!std::getline(f, line)) break;
          std::istringstream ss(line);
          float x, y, z;
          ss >> x >> y >> z;
          mesh->vertices[3 * n] = x;
          mesh->vertices[3 * n + 1] = y;
          mesh->vertices[3 * n + 2] = z;
          if (has_color) {
            uint32_t r = 0, g = 0, b = 0;
            ss >> r >> g >> b;
            mesh->colors[n] = (r << 16) | (g << 8) | b;
          }
        }
      }
    } else {
      for (uint64_t n = 0; n < nf; ++n) {
        uint32_t cnt, a, b, c;
        if (format == 1) {
          cnt = readUIntLE(f, plySize(ltype));
          int ib = plySize(itype);
          a = readUIntLE(f, ib);
          b = readUIntLE(f, ib);
          c = readUIntLE(f, ib);
        } else {
          if (!std::getline(f, line)) break;
          std::istringstream ss(line);
          ss >> cnt >> a >> b >> c;
        }
        if (cnt != 3) throw std::runtime_error(filename + ": only triangle faces are supported");
        mesh->faces[3 * n] = a;
        mesh->faces[3 * n + 1] = b;
        mesh->faces[3 * n + 2] = c;
      }
    }
  }
  if (!f) throw std::runtime_error(filename + ": truncated ply file");
  for (uint64_t i = 0; i < 3 * nf; ++i)
    if (mesh->faces[i] >= nv) throw std::runtime_error(filename + ": face index out of range");
}

void loadDomainMesh(const Domain& d, Mesh* mesh) {
  readPly(d.filename, mesh);
  if (!d.transform.isIdentity()) {
    size_t nv = mesh->vertices.size() / 3;
    for (size_t n = 0; n < nv; ++n) {
      float in[3] = {mesh->vertices[3 * n], mesh->vertices[3 * n + 1], mesh->vertices[3 * n + 2]};
      transformPoint(d.transform, in, &mesh->vertices[3 * n]);
    }
  }
}

void writePly(const std::string& filename, const float* v, uint64_t nv,
              const uint32_t* colors, const uint32_t* f, uint64_t nf) {
  std::ofstream out(filename, std::ios::out | std::ios::binary | std::ios::trunc);
  if (!out.is_open()) throw std::runtime_error("unable to write " + filename);
  out << "ply\nformat binary_little_endian 1.0\ncomment spray_gb300 wavelet isosurface\n";
  out << "element vertex " << nv << "\nproperty float x\nproperty float y\nproperty float z\n";
  out << "property uchar red\nproperty uchar green\nproperty uchar blue\n";
  out << "element face " << nf << "\nproperty list uchar int vertex_indices\nend_header\n";
  std::vector<char> buf;
  buf.reserve(nv * 15 + nf * 13);
  for (uint64_t i = 0; i < nv; ++i) {
    const char* p = (const char*)(v + 3 * i);
    buf.insert(buf.end(), p, p + 12);
    uint32_t c = colors ? colors[i] : 0u;
    buf.push_back((char)((c >> 16) & 0xff));
    buf.push_back((char)((c >> 8) & 0xff));
    buf.push_back((char)(c & 0xff));
  }
  for (uint64_t i = 0; i < nf; ++i) {
    buf.push_back(3);
    const char* p = (const char*)(f + 3 * i);
    buf.insert(buf.end(), p, p + 12);
  }
  out.write(buf.data(), (std::streamsize)buf.size());
}

// ---------------------------------------------------------------- generator
namespace {

double waveletField(double x, double y, double z, const double ph[3]) {
  return 255.0 * std::exp(-(x * x + y * y + z * z) / (2.0 * 0.5 * 0.5)) +
         10.0 * std::sin(60.0 * x + ph[0]) + 18.0 * std::sin(30.0 * y + ph[1]) +
         5.0 * std::cos(40.0 * z + ph[2]);
}

struct CubeTopology {
  // corner c = x | y<<1 | z<<2; edge e joins corners ec[e][0] -> ec[e][1]
  int ec[12][2];
  int eaxis[12];
  // face corners, counter-clockwise seen from outside the cube
  int fc[6][4];
  int edgeOf[8][8];
  CubeTopology() {
    int e = 0;
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 8; ++c)
        if (!(c & (1 << a))) {
          ec[e][0] = c;
          ec[e][1] = c | (1 << a);
          eaxis[e] = a;
          ++e;
        }
    for (int i = 0; i < 8; ++i)
      for (int j = 0; j < 8; ++j) edgeOf[i][j] = -1;
    for (int k = 0; k < 12; ++k) {
      edgeOf[ec[k][0]][ec[k][1]] = k;
      edgeOf[ec[k][1]][ec[k][0]] = k;
    }
    int fi = 0;
    for (int a = 0; a < 3; ++a) {
      int b = (a + 1) % 3, c = (a + 2) % 3;
      for (int s = 0; s < 2; ++s) {
        // (b,c) cycle (0,0)->(1,0)->(1,1)->(0,1) turns counter-clockwise about +a
        const int cyc[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
        int corners[4];
        for (int k = 0; k < 4; ++k)
          corners[k] = (s << a) | (cyc[k][0] << b) | (cyc[k][1] << c);
        for (int k = 0; k < 4; ++k) fc[fi][k] = s ? corners[k] : corners[3 - k];
        ++fi;
      }
    }
  }
};

const CubeTopology& topo() {
  static CubeTopology t;
  return t;
}

}  // namespace

void generateWavelet(const WaveletSpec& spec, std::vector<float>* vertices,
                     std::vector<uint32_t>* faces) {
  const int n = spec.samples;
  if (n < 2) throw std::runtime_error("wavelet grid needs at least 2 samples per axis");
  const double h = 2.0 / (n - 1);
  const CubeTopology& T = topo();
  std::vector<double> val((size_t)n * n * n);
  auto idx = [n](int i, int j, int k) { return ((size_t)k * n + j) * n + i; };
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        val[idx(i, j, k)] = waveletField(-1.0 + i * h, -1.0 + j * h, -1.0 + k * h, spec.phase);
  // vertex index per grid edge, one array per axis
  std::vector<int32_t> evert[3];
  for (int a = 0; a < 3; ++a) evert[a].assign((size_t)n * n * n, -1);
  vertices->clear();
  faces->clear();
  const double iso = spec.iso;
  auto edgeVertex = [&](int i, int j, int k, int a) -> uint32_t {
    int32_t& slot = evert[a][idx(i, j, k)];
    if (slot >= 0) return (uint32_t)slot;
    int i1 = i + (a == 0), j1 = j + (a == 1), k1 = k + (a == 2);
    double f0 = val[idx(i, j, k)], f1 = val[idx(i1, j1, k1)];
    double t = (iso - f0) / (f1 - f0);
    double p0[3] = {-1.0 + i * h, -1.0 + j * h, -1.0 + k * h};
    double p1[3] = {-1.0 + i1 * h, -1.0 + j1 * h, -1.0 + k1 * h};
    slot = (int32_t)(vertices->size() / 3);
    for (int c = 0; c < 3; ++c) vertices->push_back((float)(p0[c] + t * (p1[c] - p0[c])));
    return (uint32_t)slot;
  };
  for (int k = 0; k + 1 < n; ++k)
    for (int j = 0; j + 1 < n; ++j)
      for (int i = 0; i + 1 < n; ++i) {
        double cv[8];
        int inside = 0;
        for (int c = 0; c < 8; ++c) {
          cv[c] = val[idx(i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1))];
          if (cv[c] > iso) inside |= 1 << c;
        }
        if (inside == 0 || inside == 255) continue;
        int next[12];
        for (int e = 0; e < 12; ++e) next[e] = -1;
        for (int fi = 0; fi < 6; ++fi) {
          const int* q = T.fc[fi];
          int outX[2], inX[2], no = 0, ni = 0;
          for (int s = 0; s < 4; ++s) {
            int a = q[s], b = q[(s + 1) & 3];
            bool ia = (inside >> a) & 1, ib = (inside >> b) & 1;
            if (ia && !ib) outX[no++] = s;
            if (!ia && ib) inX[ni++] = s;
          }
          if (no == 0) continue;
          auto eid = [&](int s) { return T.edgeOf[q[s]][q[(s + 1) & 3]]; };
          if (no == 1) {
            next[eid(outX[0])] = eid(inX[0]);
          } else {
            // ambiguous face: mean of the corner values, summed in sorted order
            double v4[4] = {cv[q[0]], cv[q[1]], cv[q[2]], cv[q[3]]};
            std::sort(v4, v4 + 4);
            bool center_in = ((v4[0] + v4[1]) + (v4[2] + v4[3])) * 0.25 > iso;
            // out-crossing s leaves corner q[s]; in-crossing enters q[s+1]
            for (int m = 0; m < 2; ++m) {
              int so = outX[m];
              int partner;
              if (center_in) {
                // cut off the outside corner q[so+1]: its leaving edge is the
                // in-crossing at position so+1
                partner = (so + 1) & 3;
              } else {
                // cut off the inside corner q[so]: its entering edge is the
                // in-crossing at position so-1
                partner = (so + 3) & 3;
              }
              next[eid(so)] = eid(partner);
            }
          }
        }
        uint32_t vid[12];
        bool used[12] = {false};
        for (int e = 0; e < 12; ++e)
          if (next[e] >= 0) {
            int a = T.eaxis[e];
            int c0 = T.ec[e][0];
            vid[e] = edgeVertex(i + (c0 & 1), j + ((c0 >> 1) & 1), k + ((c0 >> 2) & 1), a);
          }
        for (int e = 0; e < 12; ++e) {
          if (next[e] < 0 || used[e]) continue;
          int loop[12], len = 0;
          int cur = e;
          while (!used[cur]) {
            used[cur] = true;
            loop[len++] = cur;
            cur = next[cur];
            if (cur < 0 || len > 12) throw std::runtime_error("wavelet: broken isoline loop");
          }
          for (int m = 1; m + 1 < len; ++m) {
            faces->push_back(vid[loop[0]]);
            faces->push_back(vid[loop[m]]);
            faces->push_back(vid[loop[m + 1]]);
          }
        }
      }
}

}  // namespace sg
