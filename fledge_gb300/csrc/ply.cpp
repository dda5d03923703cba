// ply.cpp — PLY mesh ingestion (MakeTriangleMesh, plymesh.cpp:19-86, which
// reads through miniply): positions (x, y, z), optional normals (nx, ny, nz)
// and texture coordinates (u, v / s, t / texture_u, texture_v) of the
// "vertex" element, and the "vertex_indices" (or "vertex_index") list of the
// "face" element.  ASCII and binary (little / big endian) files.  Faces with
// more than three corners are fan-triangulated (the reference keeps only the
// first three corners of every face); other elements are skipped.  Host
// code only: the result feeds flg_bvh_build after a copy to the device.
#include <cerrno>
#include <climits>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "../../include/flg.h"

namespace {

enum class Ty { I8, U8, I16, U16, I32, U32, F32, F64, None };

Ty parse_type(const std::string &t) {
  if (t == "char" || t == "int8") return Ty::I8;
  if (t == "uchar" || t == "uint8") return Ty::U8;
  if (t == "short" || t == "int16") return Ty::I16;
  if (t == "ushort" || t == "uint16") return Ty::U16;
  if (t == "int" || t == "int32") return Ty::I32;
  if (t == "uint" || t == "uint32") return Ty::U32;
  if (t == "float" || t == "float32") return Ty::F32;
  if (t == "double" || t == "float64") return Ty::F64;
  return Ty::None;
}

int type_size(Ty t) {
  switch (t) {
    case Ty::I8: case Ty::U8: return 1;
    case Ty::I16: case Ty::U16: return 2;
    case Ty::I32: case Ty::U32: case Ty::F32: return 4;
    case Ty::F64: return 8;
    default: return 0;
  }
}

struct Prop {
  std::string name;
  Ty type = Ty::None;
  bool list = false;
  Ty count_type = Ty::None;
};

struct Elem {
  std::string name;
  int64_t count = 0;
  std::vector<Prop> props;
};

enum class Fmt { Ascii, BinLE, BinBE };

struct Reader {
  FILE *f = nullptr;
  Fmt fmt = Fmt::Ascii;
  std::string err;

  bool fail(const char *fmt_, ...) {
    char buf[256];
    va_list ap;
    va_start(ap, fmt_);
    std::vsnprintf(buf, sizeof(buf), fmt_, ap);
    va_end(ap);
    if (err.empty()) err = buf;
    return false;
  }

  // One ASCII token (whitespace separated).
  bool token(std::string &out) {
    out.clear();
    int c;
    while ((c = std::fgetc(f)) != EOF && (c == ' ' || c == '\t' || c == '\n' || c == '\r')) {
    }
    if (c == EOF) return false;
    do {
      out.push_back((char)c);
    } while ((c = std::fgetc(f)) != EOF && !(c == ' ' || c == '\t' || c == '\n' || c == '\r'));
    return true;
  }

  // Reads one scalar of type t as double (exact for every PLY integer type
  // and for float; double is kept as is).
  bool scalar(Ty t, double &v) {
    if (fmt == Fmt::Ascii) {
      std::string s;
      if (!token(s)) return fail("unexpected end of file");
      char *end = nullptr;
      errno = 0;
      v = std::strtod(s.c_str(), &end);
      if (end == s.c_str() || *end != '\0') return fail("bad number '%s'", s.c_str());
      return true;
    }
    unsigned char b[8];
    const int n = type_size(t);
    if (n == 0 || std::fread(b, 1, (size_t)n, f) != (size_t)n) return fail("unexpected end of file");
    const bool swap = fmt == Fmt::BinBE;  // files are little or big endian; hosts here are little endian
    if (swap)
      for (int i = 0; i < n / 2; ++i) std::swap(b[i], b[n - 1 - i]);
    switch (t) {
      case Ty::I8: { int8_t x; std::memcpy(&x, b, 1); v = x; break; }
      case Ty::U8: { uint8_t x; std::memcpy(&x, b, 1); v = x; break; }
      case Ty::I16: { int16_t x; std::memcpy(&x, b, 2); v = x; break; }
      case Ty::U16: { uint16_t x; std::memcpy(&x, b, 2); v = x; break; }
      case Ty::I32: { int32_t x; std::memcpy(&x, b, 4); v = x; break; }
      case Ty::U32: { uint32_t x; std::memcpy(&x, b, 4); v = x; break; }
      case Ty::F32: { float x; std::memcpy(&x, b, 4); v = x; break; }
      case Ty::F64: { double x; std::memcpy(&x, b, 8); v = x; break; }
      default: return fail("bad type");
    }
    return true;
  }
};

bool host_little_endian() {
  const uint16_t one = 1;
  unsigned char b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

int find_prop(const Elem &e, std::initializer_list<const char *> names) {
  for (const char *nm : names)
    for (size_t i = 0; i < e.props.size(); ++i)
      if (!e.props[i].list && e.props[i].name == nm) return (int)i;
  return -1;
}

void set_err(char *err, size_t err_len, const std::string &msg) {
  if (err && err_len) {
    std::strncpy(err, msg.c_str(), err_len - 1);
    err[err_len - 1] = '\0';
  }
}

}  // namespace

namespace {

int ply_read(const char *path, flg_host_mesh *out, char *err, size_t err_len, FILE **fp) {
  if (!host_little_endian()) {
    set_err(err, err_len, "big-endian hosts are not supported");
    return FLG_ERR_UNSUPPORTED;
  }
  Reader r;
  r.f = std::fopen(path, "rb");
  *fp = r.f;
  if (!r.f) {
    set_err(err, err_len, std::string("cannot open ") + path);
    return FLG_ERR_ARG;
  }
  std::vector<Elem> elems;
  bool ok = true;
  {
    // Header: lines up to end_header.
    char line[1024];
    if (!std::fgets(line, sizeof(line), r.f) || std::strncmp(line, "ply", 3) != 0) ok = r.fail("not a PLY file");
    bool have_fmt = false;
    while (ok) {
      if (!std::fgets(line, sizeof(line), r.f)) {
        ok = r.fail("header without end_header");
        break;
      }
      char a[64] = {0}, b[64] = {0}, c[64] = {0}, d[64] = {0};
      const int n = std::sscanf(line, "%63s %63s %63s %63s", a, b, c, d);
      if (n <= 0) continue;
      const std::string k = a;
      if (k == "end_header") break;
      if (k == "comment" || k == "obj_info") continue;
      if (k == "format" && n >= 2) {
        const std::string fm = b;
        if (fm == "ascii") r.fmt = Fmt::Ascii;
        else if (fm == "binary_little_endian") r.fmt = Fmt::BinLE;
        else if (fm == "binary_big_endian") r.fmt = Fmt::BinBE;
        else ok = r.fail("unknown format %s", b);
        have_fmt = true;
      } else if (k == "element" && n >= 3) {
        Elem e;
        e.name = b;
        e.count = std::strtoll(c, nullptr, 10);
        if (e.count < 0) ok = r.fail("negative element count");
        elems.push_back(e);
      } else if (k == "property" && n >= 3 && !elems.empty()) {
        Prop p;
        if (std::string(b) == "list") {
          if (n < 4) {
            ok = r.fail("bad list property");
            break;
          }
          p.list = true;
          p.count_type = parse_type(c);
          char e2[64] = {0}, nm[64] = {0};
          std::sscanf(line, "%*s %*s %*s %63s %63s", e2, nm);
          p.type = parse_type(e2);
          p.name = nm;
          if (p.count_type == Ty::None || p.type == Ty::None) ok = r.fail("bad list types");
        } else {
          p.type = parse_type(b);
          p.name = c;
          if (p.type == Ty::None) ok = r.fail("unknown property type %s", b);
        }
        elems.back().props.push_back(p);
      } else {
        ok = r.fail("unexpected header line: %s", a);
      }
    }
    if (ok && !have_fmt) ok = r.fail("no format line");
  }
  std::vector<float> pos, nrm, uv;
  std::vector<int32_t> idx;
  bool got_v = false, got_f = false;
  int64_t n_vert = 0;
  for (size_t ei = 0; ok && ei < elems.size(); ++ei) {
    const Elem &e = elems[ei];
    const bool is_v = e.name == "vertex" && !got_v;
    const bool is_f = e.name == "face" && !got_f;
    int px = -1, py = -1, pz = -1, nx = -1, ny = -1, nz = -1, tu = -1, tv = -1, fl = -1;
    if (is_v) {
      px = find_prop(e, {"x"});
      py = find_prop(e, {"y"});
      pz = find_prop(e, {"z"});
      if (px < 0 || py < 0 || pz < 0) {
        ok = r.fail("vertex element without x, y, z");
        break;
      }
      nx = find_prop(e, {"nx"});
      ny = find_prop(e, {"ny"});
      nz = find_prop(e, {"nz"});
      tu = find_prop(e, {"u", "s", "texture_u", "texture_s"});
      tv = find_prop(e, {"v", "t", "texture_v", "texture_t"});
      n_vert = e.count;
      pos.resize((size_t)(3 * e.count));
      if (nx >= 0 && ny >= 0 && nz >= 0) nrm.resize((size_t)(3 * e.count));
      if (tu >= 0 && tv >= 0) uv.resize((size_t)(2 * e.count));
    }
    if (is_f) {
      for (size_t i = 0; i < e.props.size(); ++i)
        if (e.props[i].list && (e.props[i].name == "vertex_indices" || e.props[i].name == "vertex_index"))
          fl = (int)i;
      if (fl < 0) {
        ok = r.fail("face element without vertex_indices");
        break;
      }
    }
    std::vector<double> vals(e.props.size());
    std::vector<int64_t> corners;
    for (int64_t row = 0; ok && row < e.count; ++row) {
      for (size_t pi = 0; ok && pi < e.props.size(); ++pi) {
        const Prop &p = e.props[pi];
        if (!p.list) {
          ok = r.scalar(p.type, vals[pi]);
          continue;
        }
        double cnt_d;
        if (!(ok = r.scalar(p.count_type, cnt_d))) break;
        const int64_t cnt = (int64_t)cnt_d;
        if (cnt < 0 || cnt > (1 << 20)) {
          ok = r.fail("bad list length");
          break;
        }
        const bool keep = is_f && (int)pi == fl;
        if (keep) corners.resize((size_t)cnt);
        for (int64_t j = 0; ok && j < cnt; ++j) {
          double x;
          ok = r.scalar(p.type, x);
          if (keep) corners[(size_t)j] = (int64_t)x;
        }
      }
      if (!ok) break;
      if (is_v) {
        pos[(size_t)(3 * row)] = (float)vals[px];
        pos[(size_t)(3 * row + 1)] = (float)vals[py];
        pos[(size_t)(3 * row + 2)] = (float)vals[pz];
        if (!nrm.empty()) {
          nrm[(size_t)(3 * row)] = (float)vals[nx];
          nrm[(size_t)(3 * row + 1)] = (float)vals[ny];
          nrm[(size_t)(3 * row + 2)] = (float)vals[nz];
        }
        if (!uv.empty()) {
          uv[(size_t)(2 * row)] = (float)vals[tu];
          uv[(size_t)(2 * row + 1)] = (float)vals[tv];
        }
      }
      if (is_f) {
        if (corners.size() < 3) continue;  // degenerate face: no triangle
        for (size_t k = 1; k + 1 < corners.size(); ++k) {  // fan
          const int64_t c3[3] = {corners[0], corners[k], corners[k + 1]};
          for (int q = 0; q < 3; ++q) {
            if (c3[q] < 0 || c3[q] > INT32_MAX) {
              ok = r.fail("vertex index out of range");
              break;
            }
            idx.push_back((int32_t)c3[q]);
          }
          if (!ok) break;
        }
      }
    }
    if (is_v) got_v = ok;
    if (is_f) got_f = ok;
  }
  std::fclose(r.f);
  *fp = nullptr;
  if (ok && (!got_v || !got_f)) ok = r.fail("file has no vertex or no face element");
  if (ok) {
    for (int32_t i : idx)
      if ((int64_t)i >= n_vert) {
        ok = r.fail("face refers to vertex %d of %lld", i, (long long)n_vert);
        break;
      }
  }
  if (!ok) {
    set_err(err, err_len, r.err);
    return FLG_ERR_ARG;
  }
  auto dup = [](const auto &v) -> void * {
    if (v.empty()) return nullptr;
    void *p = std::malloc(v.size() * sizeof(v[0]));
    if (p) std::memcpy(p, v.data(), v.size() * sizeof(v[0]));
    return p;
  };
  out->pos = (float *)dup(pos);
  out->normal = (float *)dup(nrm);
  out->uv = (float *)dup(uv);
  out->idx = (int32_t *)dup(idx);
  out->n_vert = n_vert;
  out->n_tri = (int64_t)(idx.size() / 3);
  if ((n_vert > 0 && !out->pos) || (!idx.empty() && !out->idx)) {
    flg_host_mesh_free(out);
    set_err(err, err_len, "out of host memory");
    return FLG_ERR_OOM;
  }
  return FLG_OK;
}

}  // namespace

FLG_API int flg_ply_read(const char *path, flg_host_mesh *out, char *err, size_t err_len) {
  if (!path || !out) return FLG_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  FILE *fp = nullptr;
  try {
    return ply_read(path, out, err, err_len, &fp);
  } catch (...) {  // an element count too large for host memory
    if (fp) std::fclose(fp);
    flg_host_mesh_free(out);
    set_err(err, err_len, "out of host memory");
    return FLG_ERR_OOM;
  }
}

FLG_API void flg_host_mesh_free(flg_host_mesh *m) {
  if (!m) return;
  std::free(m->pos);
  std::free(m->normal);
  std::free(m->uv);
  std::free(m->idx);
  std::memset(m, 0, sizeof(*m));
}
