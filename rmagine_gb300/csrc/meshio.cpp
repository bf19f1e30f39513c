// Triangle-mesh file input/output without Assimp: PLY (ascii, binary little-
// and big-endian), Wavefront OBJ and STL (binary and ascii), plus a binary
// little-endian PLY writer.
//
// Stands in for rmagine's AssimpIO::ReadFile (map/AssimpIO.hpp:50-66, used by
// import_embree_map, EmbreeMap.hpp:94-117, and import_optix_map) for the mesh
// formats maps are stored in.  The reader returns one vertex array, one face
// array and a group index per face: OBJ objects / groups ("o", "g") become
// groups (the separate meshes Assimp would make of them); PLY and STL files are
// one group.  Polygons with more than three corners are split into a fan
// (v0, v_i, v_{i+1}).  STL triangles keep their three corners each (no vertex
// merging), as Assimp does without aiProcess_JoinIdenticalVertices.
// Host code only; any malformed input returns RMG_ERR_INVALID_ARG with a
// message, never reads past its buffers.
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/rmg.h"
#include "guard.h"

namespace rmg {
int fail(int status, const std::string& msg);
}

namespace {

struct MeshBuf {
  std::vector<rmg_vec3> v;
  std::vector<rmg_face> f;
  std::vector<uint32_t> g;
  uint32_t groups = 1;
};

int bad(const std::string& what) { return rmg::fail(RMG_ERR_INVALID_ARG, "mesh read: " + what); }

bool read_file(const char* path, std::string& data) {
  std::ifstream in(path, std::ios::binary);
  if (!in) return false;
  in.seekg(0, std::ios::end);
  const std::streamoff n = in.tellg();
  if (n < 0) return false;
  data.resize((size_t)n);
  in.seekg(0, std::ios::beg);
  if (n > 0) in.read(&data[0], n);
  return (bool)in || in.eof();
}

std::string lower(std::string s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

// ---- PLY ------------------------------------------------------------------
enum PlyType { P_I8, P_U8, P_I16, P_U16, P_I32, P_U32, P_F32, P_F64, P_BAD };

PlyType ply_type(const std::string& t) {
  if (t == "char" || t == "int8") return P_I8;
  if (t == "uchar" || t == "uint8") return P_U8;
  if (t == "short" || t == "int16") return P_I16;
  if (t == "ushort" || t == "uint16") return P_U16;
  if (t == "int" || t == "int32") return P_I32;
  if (t == "uint" || t == "uint32") return P_U32;
  if (t == "float" || t == "float32") return P_F32;
  if (t == "double" || t == "float64") return P_F64;
  return P_BAD;
}

struct PlyProp {
  std::string name;
  bool list = false;
  PlyType count_t = P_BAD, t = P_BAD;
};

struct PlyElem {
  std::string name;
  uint64_t n = 0;
  std::vector<PlyProp> props;
};

// Binary cursor with bounds checks and endianness.
struct Cursor {
  const unsigned char* p;
  size_t left;
  bool big;
  bool ok = true;
  bool take(void* dst, size_t n) {
    if (n > left) { ok = false; return false; }
    unsigned char tmp[8];
    std::memcpy(tmp, p, n);
    if (big) std::reverse(tmp, tmp + n);
    std::memcpy(dst, tmp, n);
    p += n;
    left -= n;
    return true;
  }
  bool num(PlyType t, double& out) {
    switch (t) {
      case P_I8: { int8_t x; if (!take(&x, 1)) return false; out = x; return true; }
      case P_U8: { uint8_t x; if (!take(&x, 1)) return false; out = x; return true; }
      case P_I16: { int16_t x; if (!take(&x, 2)) return false; out = x; return true; }
      case P_U16: { uint16_t x; if (!take(&x, 2)) return false; out = x; return true; }
      case P_I32: { int32_t x; if (!take(&x, 4)) return false; out = x; return true; }
      case P_U32: { uint32_t x; if (!take(&x, 4)) return false; out = x; return true; }
      case P_F32: { float x; if (!take(&x, 4)) return false; out = x; return true; }
      case P_F64: { double x; if (!take(&x, 8)) return false; out = x; return true; }
      default: ok = false; return false;
    }
  }
};

// Whitespace tokens of the ascii body.
struct Tokens {
  const char* p;
  const char* end;
  bool next(std::string& tok) {
    while (p < end && std::isspace((unsigned char)*p)) ++p;
    if (p >= end) return false;
    const char* s = p;
    while (p < end && !std::isspace((unsigned char)*p)) ++p;
    tok.assign(s, p);
    return true;
  }
  bool num(double& out) {
    std::string t;
    if (!next(t)) return false;
    char* e = nullptr;
    out = std::strtod(t.c_str(), &e);
    return e && *e == '\0';
  }
};

bool is_vertex_index_name(const std::string& n) { return n == "vertex_indices" || n == "vertex_index"; }

int add_polygon(MeshBuf& m, const std::vector<int64_t>& idx, uint32_t group) {
  if (idx.size() < 3) return RMG_OK;  // degenerate polygons are skipped
  for (size_t k = 1; k + 1 < idx.size(); ++k) {
    const int64_t a = idx[0], b = idx[k], c = idx[k + 1];
    if (a < 0 || b < 0 || c < 0 || a > 0xffffffffll || b > 0xffffffffll || c > 0xffffffffll)
      return bad("face index out of range");
    m.f.push_back(rmg_face{(uint32_t)a, (uint32_t)b, (uint32_t)c});
    m.g.push_back(group);
  }
  return RMG_OK;
}

int read_ply(const std::string& data, MeshBuf& m) {
  const size_t hdr_end_tag = data.find("end_header");
  if (data.compare(0, 3, "ply") != 0 || hdr_end_tag == std::string::npos) return bad("not a PLY file");
  size_t body = data.find('\n', hdr_end_tag);
  if (body == std::string::npos) return bad("PLY header not terminated");
  ++body;
  std::istringstream hs(data.substr(0, hdr_end_tag));
  std::string line;
  int format = -1;  // 0 ascii, 1 binary le, 2 binary be
  std::vector<PlyElem> elems;
  while (std::getline(hs, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    std::istringstream ls(line);
    std::string kw;
    ls >> kw;
    if (kw == "format") {
      std::string f;
      ls >> f;
      format = f == "ascii" ? 0 : (f == "binary_little_endian" ? 1 : (f == "binary_big_endian" ? 2 : -1));
      if (format < 0) return bad("unknown PLY format " + f);
    } else if (kw == "element") {
      PlyElem e;
      ls >> e.name >> e.n;
      if (!ls) return bad("bad PLY element line");
      elems.push_back(e);
    } else if (kw == "property") {
      if (elems.empty()) return bad("PLY property before element");
      PlyProp p;
      std::string t;
      ls >> t;
      if (t == "list") {
        std::string ct, it;
        ls >> ct >> it >> p.name;
        p.list = true;
        p.count_t = ply_type(ct);
        p.t = ply_type(it);
        if (p.count_t == P_BAD || p.t == P_BAD || p.count_t == P_F32 || p.count_t == P_F64)
          return bad("bad PLY list property");
      } else {
        p.t = ply_type(t);
        ls >> p.name;
        if (p.t == P_BAD) return bad("bad PLY property type " + t);
      }
      elems.back().props.push_back(p);
    }
  }
  if (format < 0) return bad("PLY format line missing");
  const char* b0 = data.data() + body;
  const size_t blen = data.size() - body;
  Cursor cur{reinterpret_cast<const unsigned char*>(b0), blen, format == 2};
  Tokens tok{b0, b0 + blen};
  auto get = [&](PlyType t, double& out) { return format == 0 ? tok.num(out) : cur.num(t, out); };
  std::vector<int64_t> idx;
  for (const PlyElem& e : elems) {
    const bool is_v = e.name == "vertex", is_f = e.name == "face";
    int ix = -1, iy = -1, iz = -1, ifl = -1;
    for (size_t k = 0; k < e.props.size(); ++k) {
      const auto& p = e.props[k];
      if (is_v && !p.list) {
        if (p.name == "x") ix = (int)k;
        if (p.name == "y") iy = (int)k;
        if (p.name == "z") iz = (int)k;
      }
      if (is_f && p.list && is_vertex_index_name(p.name)) ifl = (int)k;
    }
    if (is_v && (ix < 0 || iy < 0 || iz < 0)) return bad("PLY vertex element lacks x, y or z");
    if (is_v) {
      if (e.n > 0xffffffffull) return bad("too many vertices");
      m.v.reserve((size_t)e.n);
    }
    if (is_f && ifl < 0) return bad("PLY face element lacks vertex_indices");
    for (uint64_t i = 0; i < e.n; ++i) {
      double xyz[3] = {0, 0, 0};
      for (size_t k = 0; k < e.props.size(); ++k) {
        const auto& p = e.props[k];
        if (p.list) {
          double cnt;
          if (!get(p.count_t, cnt) || cnt < 0 || cnt > 1e6) return bad("truncated or bad PLY list");
          const int64_t c = (int64_t)cnt;
          if ((int)k == ifl) idx.assign((size_t)c, 0);
          for (int64_t j = 0; j < c; ++j) {
            double x;
            if (!get(p.t, x)) return bad("truncated PLY list");
            if ((int)k == ifl) idx[(size_t)j] = (int64_t)x;
          }
        } else {
          double x;
          if (!get(p.t, x)) return bad("truncated PLY body");
          if ((int)k == ix) xyz[0] = x;
          if ((int)k == iy) xyz[1] = x;
          if ((int)k == iz) xyz[2] = x;
        }
      }
      if (is_v) m.v.push_back(rmg_vec3{(float)xyz[0], (float)xyz[1], (float)xyz[2]});
      if (is_f) {
        const int s = add_polygon(m, idx, 0);
        if (s != RMG_OK) return s;
      }
    }
  }
  return RMG_OK;
}

// ---- OBJ ------------------------------------------------------------------
int read_obj(const std::string& data, MeshBuf& m) {
  size_t pos = 0;
  uint32_t group = 0;
  bool group_has_faces = false;
  std::vector<int64_t> idx;
  while (pos < data.size()) {
    size_t eol = data.find('\n', pos);
    if (eol == std::string::npos) eol = data.size();
    const char* s = data.data() + pos;
    const char* e = data.data() + eol;
    pos = eol + 1;
    while (s < e && std::isspace((unsigned char)*s)) ++s;
    if (s >= e || *s == '#') continue;
    Tokens t{s, e};
    std::string kw;
    t.next(kw);
    if (kw == "v") {
      double x, y, z;
      if (!t.num(x) || !t.num(y) || !t.num(z)) return bad("bad OBJ vertex line");
      if (m.v.size() >= 0xffffffffull) return bad("too many vertices");
      m.v.push_back(rmg_vec3{(float)x, (float)y, (float)z});
    } else if (kw == "f") {
      idx.clear();
      std::string tk;
      while (t.next(tk)) {
        char* end = nullptr;
        const long long i = std::strtoll(tk.c_str(), &end, 10);
        if (end == tk.c_str() || i == 0) return bad("bad OBJ face index '" + tk + "'");
        // 1-based; negative = relative to the vertices read so far
        idx.push_back(i > 0 ? (int64_t)i - 1 : (int64_t)m.v.size() + (int64_t)i);
      }
      for (int64_t i : idx)
        if (i < 0 || (uint64_t)i >= m.v.size()) return bad("OBJ face refers to a vertex not yet defined");
      const int st = add_polygon(m, idx, group);
      if (st != RMG_OK) return st;
      group_has_faces = true;
    } else if (kw == "o" || kw == "g") {
      if (group_has_faces) {
        ++group;
        group_has_faces = false;
      }
    }
  }
  m.groups = group + 1;
  return RMG_OK;
}

// ---- STL ------------------------------------------------------------------
int read_stl(const std::string& data, MeshBuf& m) {
  if (data.size() >= 84) {
    uint32_t n;
    std::memcpy(&n, data.data() + 80, 4);
    if ((uint64_t)84 + 50ull * n == data.size()) {
      if (3ull * n > 0xffffffffull) return bad("too many STL triangles");
      m.v.reserve(3ull * n);
      for (uint32_t i = 0; i < n; ++i) {
        const char* r = data.data() + 84 + 50ull * i + 12;  // skip the facet normal
        for (int k = 0; k < 3; ++k) {
          float xyz[3];
          std::memcpy(xyz, r + 12 * k, 12);
          m.v.push_back(rmg_vec3{xyz[0], xyz[1], xyz[2]});
        }
        m.f.push_back(rmg_face{3 * i, 3 * i + 1, 3 * i + 2});
        m.g.push_back(0);
      }
      return RMG_OK;
    }
  }
  if (lower(data.substr(0, 5)) != "solid") return bad("not an STL file");
  Tokens t{data.data(), data.data() + data.size()};
  std::string tk;
  uint32_t in_facet = 0;
  while (t.next(tk)) {
    if (tk == "vertex") {
      double x, y, z;
      if (!t.num(x) || !t.num(y) || !t.num(z)) return bad("bad STL vertex");
      m.v.push_back(rmg_vec3{(float)x, (float)y, (float)z});
      ++in_facet;
    } else if (tk == "endloop") {
      if (in_facet != 3) return bad("STL facet without three vertices");
      const uint32_t b = (uint32_t)m.v.size() - 3;
      m.f.push_back(rmg_face{b, b + 1, b + 2});
      m.g.push_back(0);
      in_facet = 0;
    }
  }
  return RMG_OK;
}

template <typename T>
T* copy_out(const std::vector<T>& v) {
  if (v.empty()) return nullptr;
  T* p = static_cast<T*>(std::malloc(sizeof(T) * v.size()));
  if (p) std::memcpy(p, v.data(), sizeof(T) * v.size());
  return p;
}

}  // namespace

extern "C" int rmg_mesh_read(const char* path, rmg_mesh* out) {
  return rmg::guarded("rmg_mesh_read", [&]() -> int {
    if (!path || !out) return rmg::fail(RMG_ERR_INVALID_ARG, "rmg_mesh_read: NULL argument");
    std::memset(out, 0, sizeof(*out));
    std::string data;
    if (!read_file(path, data)) return rmg::fail(RMG_ERR_INVALID_ARG, std::string("rmg_mesh_read: cannot read ") + path);
    const std::string p = lower(path);
    auto ends = [&](const char* ext) {
      const size_t n = std::strlen(ext);
      return p.size() >= n && p.compare(p.size() - n, n, ext) == 0;
    };
    MeshBuf m;
    int s;
    if (ends(".ply")) s = read_ply(data, m);
    else if (ends(".obj")) s = read_obj(data, m);
    else if (ends(".stl")) s = read_stl(data, m);
    else return rmg::fail(RMG_ERR_UNSUPPORTED, "rmg_mesh_read: file type not supported (.ply, .obj, .stl)");
    if (s != RMG_OK) return s;
    for (const rmg_face& f : m.f)
      if (f.v0 >= m.v.size() || f.v1 >= m.v.size() || f.v2 >= m.v.size()) return bad("face index out of range");
    out->vertices = copy_out(m.v);
    out->faces = copy_out(m.f);
    out->face_group = copy_out(m.g);
    if ((!m.v.empty() && !out->vertices) || (!m.f.empty() && (!out->faces || !out->face_group))) {
      rmg_mesh_free(out);
      return rmg::fail(RMG_ERR_OOM, "rmg_mesh_read: host allocation");
    }
    out->n_vertices = (uint32_t)m.v.size();
    out->n_faces = (uint32_t)m.f.size();
    out->n_groups = m.f.empty() ? 0 : m.groups;
    return RMG_OK;
  });
}

extern "C" void rmg_mesh_free(rmg_mesh* m) {
  if (!m) return;
  std::free(m->vertices);
  std::free(m->faces);
  std::free(m->face_group);
  std::memset(m, 0, sizeof(*m));
}

extern "C" int rmg_mesh_write_ply(const char* path, const rmg_vec3* vertices, uint32_t n_vertices,
                                  const rmg_face* faces, uint32_t n_faces) {
  return rmg::guarded("rmg_mesh_write_ply", [&]() -> int {
    if (!path || (n_vertices && !vertices) || (n_faces && !faces))
      return rmg::fail(RMG_ERR_INVALID_ARG, "rmg_mesh_write_ply: NULL argument");
    for (uint32_t i = 0; i < n_faces; ++i)
      if (faces[i].v0 >= n_vertices || faces[i].v1 >= n_vertices || faces[i].v2 >= n_vertices)
        return rmg::fail(RMG_ERR_INVALID_ARG, "rmg_mesh_write_ply: face index out of range");
    FILE* fp = std::fopen(path, "wb");
    if (!fp) return rmg::fail(RMG_ERR_INVALID_ARG, std::string("rmg_mesh_write_ply: cannot write ") + path);
    const uint16_t probe = 1;
    const bool little = *reinterpret_cast<const unsigned char*>(&probe) == 1;
    std::fprintf(fp, "ply\nformat %s 1.0\nelement vertex %u\nproperty float x\nproperty float y\nproperty float z\n"
                 "element face %u\nproperty list uchar uint vertex_indices\nend_header\n",
                 little ? "binary_little_endian" : "binary_big_endian", n_vertices, n_faces);
    bool ok = n_vertices == 0 || std::fwrite(vertices, sizeof(rmg_vec3), n_vertices, fp) == n_vertices;
    for (uint32_t i = 0; ok && i < n_faces; ++i) {
      const unsigned char c = 3;
      ok = std::fwrite(&c, 1, 1, fp) == 1 && std::fwrite(&faces[i], sizeof(rmg_face), 1, fp) == 1;
    }
    ok = (std::fclose(fp) == 0) && ok;
    return ok ? RMG_OK : rmg::fail(RMG_ERR_INVALID_ARG, "rmg_mesh_write_ply: write failed");
  });
}
