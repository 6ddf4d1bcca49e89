// NPY writer/reader for checkpoints in the reference's save layout.
#include "npy.h"

#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <sys/stat.h>
#include <sys/types.h>

namespace sns {

static const char kMagic[] = "\x93NUMPY";

static std::string npy_dict(const char *dtype, int ndim, const size_t *shape) {
  std::string s = "{'descr':";
  s += dtype;
  s += ",'fortran_order':False,'shape':(";
  for (int i = 0; i < ndim; i++) {
    s += std::to_string(shape[i]);
    s += ",";
  }
  s += ")}";
  return s;
}

int npy_write(const char *path, const char *dtype, int ndim, const size_t *shape, const void *data, size_t nbytes,
              std::string *err) {
  const std::string dict = npy_dict(dtype, ndim, shape);
  // version 1.0 stores the header length in 2 bytes, 2.0 in 4 (src/simple_npyio.c:1114-1150)
  const bool v2 = dict.size() > 65535u - 64u;
  const size_t len_bytes = v2 ? 4 : 2;
  const size_t fixed = 6 + 2 + len_bytes + dict.size();
  size_t total = 0;
  while (total <= fixed) total += 64;  // at least one padding byte: the final newline
  const size_t pad = total - fixed;
  std::vector<unsigned char> h;
  h.reserve(total);
  h.insert(h.end(), kMagic, kMagic + 6);
  h.push_back(v2 ? 2 : 1);
  h.push_back(0);
  const uint32_t hl = (uint32_t)(dict.size() + pad);
  for (size_t b = 0; b < len_bytes; b++) h.push_back((unsigned char)((hl >> (8 * b)) & 0xffu));
  h.insert(h.end(), dict.begin(), dict.end());
  h.insert(h.end(), pad - 1, (unsigned char)' ');
  h.push_back((unsigned char)'\n');
  FILE *fp = std::fopen(path, "wb");
  if (!fp) {
    if (err) *err = std::string("cannot create ") + path + ": " + std::strerror(errno);
    return 1;
  }
  bool ok = std::fwrite(h.data(), 1, h.size(), fp) == h.size();
  if (nbytes) ok = ok && std::fwrite(data, 1, nbytes, fp) == nbytes;
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok && err) *err = std::string("write failed: ") + path;
  return ok ? 0 : 1;
}

static std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t"), b = s.find_last_not_of(" \t");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// value text of key k in a python-literal dict (the reference's or numpy's spelling)
static bool dict_value(const std::string &d, const char *k, std::string *out) {
  const std::string key = std::string("'") + k + "'";
  size_t p = d.find(key);
  if (p == std::string::npos) return false;
  p = d.find(':', p + key.size());
  if (p == std::string::npos) return false;
  p = d.find_first_not_of(" \t", p + 1);
  if (p == std::string::npos) return false;
  size_t e;
  if (d[p] == '(') {
    e = d.find(')', p);
    if (e == std::string::npos) return false;
    *out = d.substr(p, e - p + 1);
  } else {
    e = d.find_first_of(",}", p);
    if (e == std::string::npos) return false;
    *out = trim(d.substr(p, e - p));
  }
  return true;
}

int npy_read(const char *path, const char *dtype, int ndim, const size_t *shape, void *data, size_t nbytes,
             std::string *err) {
  FILE *fp = std::fopen(path, "rb");
  if (!fp) {
    if (err) *err = std::string("cannot open ") + path + ": " + std::strerror(errno);
    return 1;
  }
  auto bad = [&](const std::string &why) {
    std::fclose(fp);
    if (err) *err = std::string(path) + ": " + why;
    return 1;
  };
  unsigned char pre[8];
  if (std::fread(pre, 1, 8, fp) != 8 || std::memcmp(pre, kMagic, 6) != 0) return bad("not an NPY file");
  const int major = pre[6];
  if (major != 1 && major != 2 && major != 3) return bad("unsupported NPY version");
  const size_t len_bytes = major == 1 ? 2 : 4;
  unsigned char lb[4] = {0, 0, 0, 0};
  if (std::fread(lb, 1, len_bytes, fp) != len_bytes) return bad("truncated header");
  uint32_t hl = 0;
  for (size_t b = 0; b < len_bytes; b++) hl |= (uint32_t)lb[b] << (8 * b);
  std::string dict(hl, '\0');
  if (hl && std::fread(&dict[0], 1, hl, fp) != hl) return bad("truncated header");
  std::string descr, order, shp;
  if (!dict_value(dict, "descr", &descr) || !dict_value(dict, "fortran_order", &order) ||
      !dict_value(dict, "shape", &shp))
    return bad("malformed header dictionary");
  const std::string want = dtype;
  const std::string alt = want == "'float64'" ? "'<f8'" : want == "'int32'" ? "'<i4'" : want;
  if (descr != want && descr != alt) return bad("dtype " + descr + ", expected " + want);
  if (order != "False") return bad("Fortran-ordered data is not supported");
  std::vector<size_t> dims;
  {
    std::string inner = shp.substr(1, shp.size() - 2);
    size_t p = 0;
    while (p < inner.size()) {
      size_t e = inner.find(',', p);
      const std::string tok = trim(inner.substr(p, e == std::string::npos ? std::string::npos : e - p));
      if (!tok.empty()) dims.push_back((size_t)std::stoull(tok));
      if (e == std::string::npos) break;
      p = e + 1;
    }
  }
  bool same = (int)dims.size() == ndim;
  for (int i = 0; same && i < ndim; i++) same = dims[i] == shape[i];
  if (!same) {
    std::string s = "shape " + shp + ", expected (";
    for (int i = 0; i < ndim; i++) s += std::to_string(shape[i]) + ",";
    return bad(s + ")");
  }
  if (nbytes && std::fread(data, 1, nbytes, fp) != nbytes) return bad("truncated data");
  std::fclose(fp);
  return 0;
}

int make_dirs(const char *path, std::string *err) {
  std::string p(path);
  for (size_t i = 1; i <= p.size(); i++) {
    if (i == p.size() || p[i] == '/') {
      const std::string sub = p.substr(0, i);
      if (mkdir(sub.c_str(), 0777) != 0 && errno != EEXIST) {
        if (err) *err = "cannot create directory " + sub + ": " + std::strerror(errno);
        return 1;
      }
    }
  }
  return 0;
}

}  // namespace sns
