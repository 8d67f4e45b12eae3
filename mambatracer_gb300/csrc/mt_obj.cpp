// Wavefront OBJ text to the reference's mesh arrays, the ingest path of
// TracerAPI.initMesh / TracerAPI.init (src/cl/ui/fx/main/TracerAPI.java:321-323,
// :393-438), which hands a file or string to an OBJ parser that fills CMesh
// (src/cl/scene/CMesh.java:125-157) and then calls CMesh.initCLBuffers. That
// parser lives in a library the reference does not ship; this reader follows
// the contract its callers rely on:
//   v x y z      a point (float4, w = 0)
//   vt u v       a texture coordinate (float2)
//   vn x y z     a normal (float4, w = 0)
//   f a b c ...  a polygon of v, v/vt, v//vn or v/vt/vn references (1-based;
//                negative counts back from the last element read), split into
//                a fan of triangles (a, b, c), (a, c, d), ...
//   o name, g name   a new object: each distinct name gets the next material
//                index in order of first appearance (the reference's default
//                scene numbers its materials 0 floor .. 7 left wall in the order
//                of its `o` lines, TracerAPI.java:325-335); faces before any
//                name belong to material 0
// A face's uv (normal) indices are -1 unless all its corners name one, as the
// reference's kernels test `uvx > -1` (Util.cl:270-300). `mat` holds the
// material index in its low 16 bits and the same index as the group in the
// high bits (Util.cl:11-14). Other statements (s, usemtl, mtllib, l, p) are
// read and ignored.
#include <algorithm>
#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "mambatracer.h"

namespace mt {
__attribute__((visibility("hidden"))) void set_last_error(const char* msg);
}

namespace {

struct Mesh {
  std::vector<float> points, uvs, normals;
  std::vector<int32_t> faces;
  int groups = 0;
};

bool next_token(const char*& p, const char* end, const char*& tok, size_t& n) {
  while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
  if (p >= end) return false;
  tok = p;
  while (p < end && *p != ' ' && *p != '\t' && *p != '\r') ++p;
  n = (size_t)(p - tok);
  return n > 0;
}

bool parse_float(const char* tok, size_t n, float* out) {
  char buf[64];
  if (n >= sizeof(buf)) return false;
  std::memcpy(buf, tok, n);
  buf[n] = 0;
  char* e = nullptr;
  errno = 0;
  float v = std::strtof(buf, &e);
  if (e != buf + n) return false;
  *out = v;
  return true;
}

// an OBJ index (1-based, or negative from the end) to a 0-based one; -1 when empty
bool resolve(const char* s, size_t n, size_t count, int* out) {
  if (n == 0) {
    *out = -1;
    return true;
  }
  char buf[32];
  if (n >= sizeof(buf)) return false;
  std::memcpy(buf, s, n);
  buf[n] = 0;
  char* e = nullptr;
  long v = std::strtol(buf, &e, 10);
  if (e != buf + n || v == 0) return false;
  long idx = v > 0 ? v - 1 : (long)count + v;
  if (idx < 0 || idx >= (long)count || idx > INT32_MAX) return false;
  *out = (int)idx;
  return true;
}

int parse(const char* text, size_t len, Mesh& m, std::string& err) {
  std::unordered_map<std::string, int> names;
  int group = 0;
  int base = -1;  // index of the first name: 1 when faces came before any name
  const char* p = text;
  const char* end = text + len;
  int line = 0;
  std::vector<int> cv, ct, cn;
  while (p < end) {
    ++line;
    const char* eol = static_cast<const char*>(std::memchr(p, '\n', (size_t)(end - p)));
    if (!eol) eol = end;
    const char* q = p;
    p = eol < end ? eol + 1 : end;
    const char* hash = static_cast<const char*>(std::memchr(q, '#', (size_t)(eol - q)));
    const char* lend = hash ? hash : eol;
    const char* tok;
    size_t n;
    if (!next_token(q, lend, tok, n)) continue;
    std::string kw(tok, n);
    auto bad = [&](const char* what) {
      err = "OBJ line " + std::to_string(line) + ": " + what;
      return MT_ERR_INVALID;
    };
    if (kw == "v" || kw == "vn") {
      float xyz[3];
      for (int k = 0; k < 3; ++k)
        if (!next_token(q, lend, tok, n) || !parse_float(tok, n, &xyz[k])) return bad("bad coordinate");
      auto& dst = kw == "v" ? m.points : m.normals;
      dst.insert(dst.end(), {xyz[0], xyz[1], xyz[2], 0.f});
    } else if (kw == "vt") {
      float uv[2];
      for (int k = 0; k < 2; ++k)
        if (!next_token(q, lend, tok, n) || !parse_float(tok, n, &uv[k])) return bad("bad texture coordinate");
      m.uvs.insert(m.uvs.end(), {uv[0], uv[1]});
    } else if (kw == "o" || kw == "g") {
      const char* nt;
      size_t nn;
      std::string name = next_token(q, lend, nt, nn) ? std::string(nt, (size_t)(lend - nt)) : std::string();
      while (!name.empty() && (name.back() == ' ' || name.back() == '\t' || name.back() == '\r')) name.pop_back();
      if (base < 0) base = m.faces.empty() ? 0 : 1;  // earlier faces keep material 0 to themselves
      auto it = names.find(name);
      if (it == names.end()) it = names.emplace(name, base + (int)names.size()).first;
      group = it->second;
      if (group > 0xFFFF) return bad("more than 65536 objects (16-bit material index)");
    } else if (kw == "f") {
      cv.clear();
      ct.clear();
      cn.clear();
      while (next_token(q, lend, tok, n)) {
        const char* s1 = static_cast<const char*>(std::memchr(tok, '/', n));
        size_t nv = s1 ? (size_t)(s1 - tok) : n;
        int v = -1, t = -1, nr = -1;
        if (!resolve(tok, nv, m.points.size() / 4, &v) || v < 0) return bad("bad vertex index");
        if (s1) {
          const char* r = s1 + 1;
          const char* rend = tok + n;
          const char* s2 = static_cast<const char*>(std::memchr(r, '/', (size_t)(rend - r)));
          size_t nt2 = s2 ? (size_t)(s2 - r) : (size_t)(rend - r);
          if (!resolve(r, nt2, m.uvs.size() / 2, &t)) return bad("bad texture index");
          if (s2 && !resolve(s2 + 1, (size_t)(rend - s2 - 1), m.normals.size() / 4, &nr)) return bad("bad normal index");
        }
        cv.push_back(v);
        ct.push_back(t);
        cn.push_back(nr);
      }
      if (cv.size() < 3) return bad("a face needs three corners");
      bool all_t = true, all_n = true;
      for (size_t k = 0; k < cv.size(); ++k) {
        all_t = all_t && ct[k] >= 0;
        all_n = all_n && cn[k] >= 0;
      }
      for (size_t k = 1; k + 1 < cv.size(); ++k) {
        const size_t c[3] = {0, k, k + 1};
        int32_t f[10];
        for (int j = 0; j < 3; ++j) {
          f[j] = cv[c[j]];
          f[3 + j] = all_t ? ct[c[j]] : -1;
          f[6 + j] = all_n ? cn[c[j]] : -1;
        }
        f[9] = (int32_t)(((uint32_t)group << 16) | (uint32_t)group);
        m.faces.insert(m.faces.end(), f, f + 10);
        if (m.faces.size() / 10 > (size_t)INT32_MAX / 2) return bad("too many faces");
      }
    }
  }
  // material count: the largest index used + 1 (0 when there are no faces)
  int maxg = -1;
  for (size_t i = 9; i < m.faces.size(); i += 10) maxg = std::max(maxg, m.faces[i] & 0xFFFF);
  m.groups = maxg + 1;
  return MT_OK;
}

}  // namespace

extern "C" int mt_obj_parse(const char* text, size_t len, int32_t* counts, float* points, float* uvs, float* normals,
                            int32_t* faces) {
  if (!text || !counts) {
    mt::set_last_error("mt_obj_parse: NULL argument");
    return MT_ERR_INVALID;
  }
  Mesh m;
  std::string err;
  int r = parse(text, len, m, err);
  if (r) {
    mt::set_last_error(err.c_str());
    return r;
  }
  const int32_t c[5] = {(int32_t)(m.points.size() / 4), (int32_t)(m.uvs.size() / 2), (int32_t)(m.normals.size() / 4),
                        (int32_t)(m.faces.size() / 10), (int32_t)m.groups};
  std::memcpy(counts, c, sizeof(c));
  if (points) std::memcpy(points, m.points.data(), m.points.size() * 4);
  if (uvs) std::memcpy(uvs, m.uvs.data(), m.uvs.size() * 4);
  if (normals) std::memcpy(normals, m.normals.data(), m.normals.size() * 4);
  if (faces) std::memcpy(faces, m.faces.data(), m.faces.size() * 4);
  return MT_OK;
}
