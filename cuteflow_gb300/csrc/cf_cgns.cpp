/*
 * cf_cgns.cpp -- CGNS/HDF5 triangle meshes (is_cgns = 1) for cf_case_read, without libcgns.
 *
 * lec_mail_cgns (maillage.cuf:398-778) reads, for one process: base 1; the zone whose ordinal is
 * the process id (0); its node and element counts (the zone's sizes); CoordinateX/Y/Z; the
 * triangle connectivity of section 1; the boundary conditions of type BCInflow (9) and BCOutflow
 * (13) with more than one node, numbered by matching their names against the namelist's
 * inlet_name / outlet_name (1 when no name matches); and the user data "Manning" (per element),
 * unless is_override_manning.  It marks no wall nodes.  The ghost-element blocks (ElemsToSend /
 * ElemsToRecv) describe an MPI partition and are not read here (one domain).
 *
 * The HDF5 container is walked directly, following the public HDF5 File Format Specification
 * (version 3.0): superblock versions 2 and 3, version-2 object headers with continuation blocks,
 * link messages of compact groups, attribute messages, and datasets with compact, contiguous or
 * chunked (version-1 B-tree index) layout of integers, floats and strings.  Filtered (compressed)
 * datasets, dense link storage and other layouts are reported as not supported.  The checksums of
 * the superblock and of every object header are verified, and every read is bounds-checked: a
 * malformed file gives an error, never a crash.  Host code only.
 */
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "cf_internal.h"

namespace cf {

namespace {

struct H5Error {
  int code;
  std::string msg;
};

[[noreturn]] void h5fail(int code, const std::string& msg) { throw H5Error{code, msg}; }

struct Msg {
  int type;
  size_t off, len;
};

/* Bob Jenkins' lookup3 hash of bytes (hashlittle, public domain, 2006), which HDF5 stores as the
 * checksum of its version-2 superblocks and object headers (initial value 0). */
uint32_t lookup3(const uint8_t* k, size_t length, uint32_t initval) {
  auto rot = [](uint32_t x, int r) { return (x << r) | (x >> (32 - r)); };
  uint32_t a, b, c;
  a = b = c = 0xdeadbeefu + (uint32_t)length + initval;
  auto word = [&](size_t i) {
    return (uint32_t)k[i] | ((uint32_t)k[i + 1] << 8) | ((uint32_t)k[i + 2] << 16) | ((uint32_t)k[i + 3] << 24);
  };
  while (length > 12) {
    a += word(0);
    b += word(4);
    c += word(8);
    a -= c; a ^= rot(c, 4);  c += b;
    b -= a; b ^= rot(a, 6);  a += c;
    c -= b; c ^= rot(b, 8);  b += a;
    a -= c; a ^= rot(c, 16); c += b;
    b -= a; b ^= rot(a, 19); a += c;
    c -= b; c ^= rot(b, 4);  b += a;
    length -= 12;
    k += 12;
  }
  if (length == 0) return c;
  uint8_t tail[12] = {0};
  std::memcpy(tail, k, length);
  a += (uint32_t)tail[0] | ((uint32_t)tail[1] << 8) | ((uint32_t)tail[2] << 16) | ((uint32_t)tail[3] << 24);
  b += (uint32_t)tail[4] | ((uint32_t)tail[5] << 8) | ((uint32_t)tail[6] << 16) | ((uint32_t)tail[7] << 24);
  c += (uint32_t)tail[8] | ((uint32_t)tail[9] << 8) | ((uint32_t)tail[10] << 16) | ((uint32_t)tail[11] << 24);
  c ^= b; c -= rot(b, 14);
  a ^= c; a -= rot(c, 11);
  b ^= a; b -= rot(a, 25);
  c ^= b; c -= rot(b, 16);
  a ^= c; a -= rot(c, 4);
  b ^= a; b -= rot(a, 14);
  c ^= b; c -= rot(b, 24);
  return c;
}

/* a * b, or an error when the product leaves 2^40 (no array of a mesh file comes near it) */
uint64_t mul_checked(uint64_t a, uint64_t b) {
  const uint64_t lim = (uint64_t)1 << 40;
  if (a > lim || b > lim || (a != 0 && b > lim / a)) h5fail(CF_EINVAL, "HDF5 dataset dimensions too large");
  return a * b;
}

struct Data {
  int cls = -1;            /* 0 integer, 1 float, 3 string */
  bool is_signed = true;
  uint32_t size = 0;       /* bytes per element */
  std::vector<uint64_t> dims;
  std::vector<uint8_t> raw;
  uint64_t count() const {
    uint64_t n = 1;
    for (uint64_t d : dims) n = mul_checked(n, d);
    return n;
  }
};

class H5 {
 public:
  explicit H5(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) h5fail(CF_EINVAL, "cannot open the CGNS mesh " + path);
    b_.assign(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    if (b_.size() < 16 || std::memcmp(b_.data(), sig, 8) != 0) h5fail(CF_EINVAL, path + " is not an HDF5 file");
    const int ver = b_[8];
    if (ver != 2 && ver != 3) h5fail(CF_ENOTSUP, "HDF5 superblock version " + std::to_string(ver) + " is not supported");
    so_ = b_[9];
    sl_ = b_[10];
    if (so_ < 1 || so_ > 8 || sl_ < 1 || sl_ > 8) h5fail(CF_EINVAL, "bad HDF5 offset/length sizes");
    size_t p = 12;
    p += so_;          /* base address */
    p += so_;          /* superblock extension */
    p += so_;          /* end of file */
    root_ = u(p, so_);
    checksum(0, p + so_, "superblock");
  }

  uint64_t root() const { return root_; }

  uint64_t u(size_t p, int n) const {
    need(p, (size_t)n);
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = (v << 8) | b_[p + i];
    return v;
  }

  /* messages of a version-2 object header, following continuation blocks */
  std::vector<Msg> messages(uint64_t addr) const {
    need(addr, 6);
    if (std::memcmp(&b_[addr], "OHDR", 4) != 0) h5fail(CF_ENOTSUP, "version-1 HDF5 object headers are not supported");
    const int flags = b_[addr + 5];
    size_t p = addr + 6;
    if (flags & 0x20) p += 16;
    if (flags & 0x10) p += 4;
    const int csize = 1 << (flags & 3);
    const uint64_t size0 = u(p, csize);
    p += csize;
    const bool track = (flags & 0x04) != 0;
    need(p, size0 + 4);
    checksum(addr, (size_t)(p - addr + size0), "object header");
    std::vector<std::pair<size_t, size_t>> chunks{{p, p + (size_t)size0}};
    std::vector<Msg> out;
    for (size_t ci = 0; ci < chunks.size(); ++ci) {
      if (ci > 64) h5fail(CF_EINVAL, "too many HDF5 header continuation blocks");
      size_t q = chunks[ci].first;
      const size_t end = chunks[ci].second;
      need(q, end - q);
      while (q + 4 <= end) {
        const int mtype = b_[q];
        const size_t msize = (size_t)u(q + 1, 2);
        q += 4 + (track ? 2 : 0);
        if (q + msize > end) break;
        if (mtype == 0x10) {   /* continuation */
          const uint64_t caddr = u(q, so_), clen = u(q + so_, sl_);
          need(caddr, clen);
          if (clen >= 8 && std::memcmp(&b_[caddr], "OCHK", 4) == 0) {
            checksum(caddr, (size_t)clen - 4, "object header continuation");
            chunks.emplace_back(caddr + 4, caddr + clen - 4);
          }
        } else if (mtype != 0) {
          out.push_back({mtype, q, msize});
        }
        q += msize;
      }
    }
    return out;
  }

  /* hard links of a compact group (name, object address), in header order */
  std::vector<std::pair<std::string, uint64_t>> links(uint64_t addr) const {
    std::vector<std::pair<std::string, uint64_t>> res;
    bool dense = false;
    for (const Msg& m : messages(addr)) {
      if (m.type == 0x02) {   /* link info: a fractal-heap address means dense storage */
        const int flags = b_[m.off + 1];
        const size_t p = m.off + 2 + ((flags & 1) ? 8 : 0);
        if (p + so_ <= m.off + m.len && u(p, so_) != ~0ull >> (64 - 8 * so_)) dense = true;
      }
      if (m.type != 0x06) continue;
      const uint8_t* d = &b_[m.off];
      const int flags = d[1];
      size_t p = 2;
      int ltype = 0;
      if (flags & 0x08) ltype = d[p++];
      if (flags & 0x04) p += 8;
      if (flags & 0x10) p += 1;
      const int ln = 1 << (flags & 3);
      if (p + ln > m.len) h5fail(CF_EINVAL, "bad HDF5 link message");
      const uint64_t nlen = u(m.off + p, ln);
      p += ln;
      if (p + nlen > m.len) h5fail(CF_EINVAL, "bad HDF5 link name");
      std::string name(reinterpret_cast<const char*>(d + p), (size_t)nlen);
      p += nlen;
      if (ltype == 0 && p + so_ <= m.len) res.emplace_back(name, u(m.off + p, so_));
    }
    if (res.empty() && dense) h5fail(CF_ENOTSUP, "HDF5 dense link storage is not supported");
    return res;
  }

  /* a string attribute, or "" */
  std::string attr_string(uint64_t addr, const char* want) const {
    for (const Msg& m : messages(addr)) {
      if (m.type != 0x0C || m.len < 8) continue;
      const uint8_t* d = &b_[m.off];
      const int ver = d[0];
      const size_t nsz = (size_t)u(m.off + 2, 2), tsz = (size_t)u(m.off + 4, 2), ssz = (size_t)u(m.off + 6, 2);
      auto pad = [&](size_t n) { return ver == 1 ? (n + 7) / 8 * 8 : n; };
      size_t p = 8 + (ver == 3 ? 1 : 0);
      if (p + pad(nsz) + pad(tsz) + pad(ssz) > m.len || tsz < 8) continue;
      const std::string name(reinterpret_cast<const char*>(d + p), strnlen(reinterpret_cast<const char*>(d + p), nsz));
      p += pad(nsz);
      const uint8_t* dt = d + p;
      p += pad(tsz) + pad(ssz);
      if (name != want || (dt[0] & 0x0F) != 3) continue;
      const size_t sz = (size_t)u((size_t)(dt - b_.data()) + 4, 4);
      const size_t n = std::min(sz, m.len - p);
      return std::string(reinterpret_cast<const char*>(d + p), strnlen(reinterpret_cast<const char*>(d + p), n));
    }
    return "";
  }

  Data dataset(uint64_t addr) const {
    Data out;
    int lclass = -1;
    std::vector<uint8_t> compact;
    uint64_t caddr = 0, clen = 0, baddr = 0;
    std::vector<uint64_t> cdims;
    for (const Msg& m : messages(addr)) {
      const uint8_t* d = &b_[m.off];
      if (m.type == 0x0B && m.len >= 2 && d[1] > 0) h5fail(CF_ENOTSUP, "filtered (compressed) HDF5 datasets are not supported");
      if (m.type == 0x01) {
        const int ver = d[0], rank = d[1];
        const size_t p = (ver == 1) ? 8 : 4;
        if (p + (size_t)rank * sl_ > m.len) h5fail(CF_EINVAL, "bad HDF5 dataspace");
        out.dims.clear();
        for (int i = 0; i < rank; ++i) out.dims.push_back(u(m.off + p + (size_t)i * sl_, sl_));
      } else if (m.type == 0x03) {
        if (m.len < 8) h5fail(CF_EINVAL, "bad HDF5 datatype");
        out.cls = d[0] & 0x0F;
        out.is_signed = (d[1] & 0x08) != 0;
        out.size = (uint32_t)u(m.off + 4, 4);
        if (out.cls != 0 && out.cls != 1 && out.cls != 3)
          h5fail(CF_ENOTSUP, "HDF5 datatype class " + std::to_string(out.cls) + " is not supported");
        if (out.cls != 3 && (d[1] & 0x01)) h5fail(CF_ENOTSUP, "big-endian HDF5 data is not supported");
      } else if (m.type == 0x08) {
        if (m.len < 2 || d[0] != 3) h5fail(CF_ENOTSUP, "HDF5 data layout version " + std::to_string(d[0]));
        lclass = d[1];
        if (lclass == 0) {
          const size_t n = (size_t)u(m.off + 2, 2);
          if (4 + n > m.len) h5fail(CF_EINVAL, "bad HDF5 compact layout");
          compact.assign(d + 4, d + 4 + n);
        } else if (lclass == 1) {
          caddr = u(m.off + 2, so_);
          clen = u(m.off + 2 + so_, sl_);
        } else if (lclass == 2) {
          const int rank1 = d[2];
          baddr = u(m.off + 3, so_);
          cdims.clear();
          for (int k = 0; k < rank1; ++k) cdims.push_back(u(m.off + 3 + so_ + 4 * (size_t)k, 4));
        } else {
          h5fail(CF_ENOTSUP, "HDF5 layout class " + std::to_string(lclass) + " is not supported");
        }
      }
    }
    if (out.cls < 0 || lclass < 0) h5fail(CF_EINVAL, "HDF5 dataset without type or layout");
    if (out.size == 0) h5fail(CF_EINVAL, "bad HDF5 element size");
    const uint64_t n = out.count(), nbytes = mul_checked(n, out.size);
    if (lclass == 0) {
      if (compact.size() < nbytes) h5fail(CF_EINVAL, "short HDF5 compact dataset");
      out.raw.assign(compact.begin(), compact.begin() + (size_t)nbytes);
    } else if (lclass == 1) {
      if (clen < nbytes) h5fail(CF_EINVAL, "short HDF5 contiguous dataset");
      need(caddr, nbytes);
      out.raw.assign(b_.begin() + (size_t)caddr, b_.begin() + (size_t)(caddr + nbytes));
    } else {
      const size_t rank = out.dims.size();
      if (cdims.size() != rank + 1) h5fail(CF_EINVAL, "bad HDF5 chunk dimensions");
      out.raw.assign((size_t)nbytes, 0);
      chunks(baddr, rank, cdims, out, 0);
    }
    return out;
  }

 private:
  void need(uint64_t p, uint64_t n) const {
    if (p > b_.size() || n > b_.size() - p) h5fail(CF_EINVAL, "HDF5 structure outside the file");
  }

  /* the lookup3 checksum stored after the n bytes at p */
  void checksum(uint64_t p, size_t n, const char* what) const {
    need(p, (uint64_t)n + 4);
    if (lookup3(&b_[p], n, 0) != (uint32_t)u(p + n, 4))
      h5fail(CF_EINVAL, std::string("HDF5 ") + what + " checksum mismatch (corrupted file)");
  }

  /* a version-1 B-tree of raw-data chunks: copy every chunk into out.raw */
  void chunks(uint64_t addr, size_t rank, const std::vector<uint64_t>& cdims, Data& out, int depth) const {
    if (depth > 32) h5fail(CF_EINVAL, "HDF5 chunk B-tree too deep");
    need(addr, 8 + 2 * (uint64_t)so_);
    if (std::memcmp(&b_[addr], "TREE", 4) != 0 || b_[addr + 4] != 1) h5fail(CF_EINVAL, "bad HDF5 chunk B-tree");
    const int level = b_[addr + 5];
    const int used = (int)u(addr + 6, 2);
    size_t p = addr + 8 + 2 * (size_t)so_;
    const size_t keysize = 8 + 8 * (rank + 1);
    for (int i = 0; i < used; ++i) {
      const uint64_t csize = u(p, 4), fmask = u(p + 4, 4);
      std::vector<uint64_t> offs(rank);
      for (size_t k = 0; k < rank; ++k) offs[k] = u(p + 8 + 8 * k, 8);
      const uint64_t child = u(p + keysize, so_);
      if (level > 0) {
        chunks(child, rank, cdims, out, depth + 1);
      } else {
        if (fmask != 0) h5fail(CF_ENOTSUP, "filtered HDF5 chunks are not supported");
        uint64_t per = out.size;
        for (size_t k = 0; k < rank; ++k) per = mul_checked(per, cdims[k]);
        if (csize < per) h5fail(CF_EINVAL, "short HDF5 chunk");
        need(child, per);
        copy_chunk(&b_[child], offs, cdims, out);
      }
      p += keysize + so_;
    }
  }

  /* place a chunk (C order, dims cdims[0..rank-1]) at offsets offs of the full array */
  static void copy_chunk(const uint8_t* src, const std::vector<uint64_t>& offs, const std::vector<uint64_t>& cdims,
                         Data& out) {
    const size_t rank = offs.size();
    std::vector<uint64_t> idx(rank, 0);
    const uint64_t es = out.size;
    uint64_t total = 1;
    for (size_t k = 0; k < rank; ++k) total = mul_checked(total, cdims[k]);
    for (uint64_t e = 0; e < total; ++e) {
      uint64_t lin = 0;
      bool inside = true;
      for (size_t k = 0; k < rank; ++k) {
        const uint64_t g = offs[k] + idx[k];
        if (g >= out.dims[k]) inside = false;
        lin = lin * out.dims[k] + g;
      }
      if (inside) std::memcpy(&out.raw[(size_t)(lin * es)], src + e * es, (size_t)es);
      for (size_t k = rank; k-- > 0;) {   /* next element, last dimension fastest */
        if (++idx[k] < cdims[k]) break;
        idx[k] = 0;
      }
    }
  }

  std::vector<uint8_t> b_;
  int so_ = 8, sl_ = 8;
  uint64_t root_ = 0;
};

/* ---- CGNS nodes on top of HDF5 -------------------------------------------------------- */

struct Node {
  std::string name;
  uint64_t addr;
};

std::vector<Node> children(const H5& h, uint64_t addr, const char* label) {
  std::vector<Node> out;
  for (const auto& l : h.links(addr)) {
    if (l.first == " data") continue;
    if (!label || h.attr_string(l.second, "label") == label) out.push_back({l.first, l.second});
  }
  return out;
}

bool child(const H5& h, uint64_t addr, const std::string& name, uint64_t& out) {
  for (const auto& l : h.links(addr))
    if (l.first == name) {
      out = l.second;
      return true;
    }
  return false;
}

bool node_data(const H5& h, uint64_t addr, Data& out) {
  uint64_t d;
  if (!child(h, addr, " data", d)) return false;
  out = h.dataset(d);
  return true;
}

std::vector<double> as_double(const Data& d, const std::string& what) {
  std::vector<double> v((size_t)d.count());
  if (d.cls == 1 && d.size == 8) {
    std::memcpy(v.data(), d.raw.data(), v.size() * 8);
  } else if (d.cls == 1 && d.size == 4) {
    for (size_t i = 0; i < v.size(); ++i) {
      float f;
      std::memcpy(&f, &d.raw[4 * i], 4);
      v[i] = f;
    }
  } else {
    h5fail(CF_EINVAL, what + ": expected real data");
  }
  return v;
}

std::vector<int64_t> as_int(const Data& d, const std::string& what) {
  std::vector<int64_t> v((size_t)d.count());
  if (d.cls != 0 || (d.size != 4 && d.size != 8)) h5fail(CF_EINVAL, what + ": expected integer data");
  for (size_t i = 0; i < v.size(); ++i) {
    if (d.size == 8) {
      int64_t x;
      std::memcpy(&x, &d.raw[8 * i], 8);
      v[i] = x;
    } else {
      int32_t x;
      std::memcpy(&x, &d.raw[4 * i], 4);
      v[i] = d.is_signed ? (int64_t)x : (int64_t)(uint32_t)x;
    }
  }
  return v;
}

std::string as_string(const Data& d) {
  std::string s(d.raw.begin(), d.raw.end());
  const size_t z = s.find('\0');
  return z == std::string::npos ? s : s.substr(0, z);
}

std::string trimmed(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  return s.substr(a, s.find_last_not_of(" \t\r\n") - a + 1);
}

}  // namespace

int read_cgns_mesh(const std::string& path, const std::vector<std::string>& inlet_names,
                   const std::vector<std::string>& outlet_names, bool want_manning, CgnsMesh& M, std::string& err) {
  try {
    H5 h(path);
    const auto bases = children(h, h.root(), "CGNSBase_t");
    if (bases.empty()) h5fail(CF_EINVAL, "no CGNS base in " + path);
    /* the zone of process 0: ordinal 0, or no ordinal */
    const auto zones = children(h, bases[0].addr, "Zone_t");
    uint64_t zone = 0;
    bool found = false;
    for (const Node& z : zones) {
      uint64_t o;
      Data od;
      if (child(h, z.addr, "Ordinal", o) && node_data(h, o, od) && as_int(od, "Ordinal")[0] != 0) continue;
      zone = z.addr;
      found = true;
      break;
    }
    if (!found) h5fail(CF_EINVAL, "no CGNS zone of ordinal 0 in " + path);
    Data zd;
    if (!node_data(h, zone, zd)) h5fail(CF_EINVAL, "CGNS zone without sizes");
    const auto sizes = as_int(zd, "zone sizes");
    if (sizes.size() < 2 || sizes[0] < 1 || sizes[1] < 1) h5fail(CF_EINVAL, "bad CGNS zone sizes");
    const int64_t nnt = sizes[0], nelt = sizes[1];
    /* coordinates */
    uint64_t gc;
    if (!child(h, zone, "GridCoordinates", gc)) h5fail(CF_EINVAL, "CGNS zone without GridCoordinates");
    const char* cn[3] = {"CoordinateX", "CoordinateY", "CoordinateZ"};
    std::vector<double>* dst[3] = {&M.x, &M.y, &M.z};
    for (int k = 0; k < 3; ++k) {
      uint64_t a;
      Data d;
      if (!child(h, gc, cn[k], a) || !node_data(h, a, d)) h5fail(CF_EINVAL, std::string("CGNS mesh without ") + cn[k]);
      *dst[k] = as_double(d, cn[k]);
      if ((int64_t)dst[k]->size() != nnt) h5fail(CF_EINVAL, std::string(cn[k]) + " does not have the zone's node count");
    }
    /* section 1: triangles */
    const auto sections = children(h, zone, "Elements_t");
    if (sections.empty()) h5fail(CF_EINVAL, "CGNS zone without element sections");
    Data sd;
    if (!node_data(h, sections[0].addr, sd)) h5fail(CF_EINVAL, "CGNS section without element type");
    const auto stype = as_int(sd, "section type");
    if (stype.empty() || stype[0] != 5) h5fail(CF_ENOTSUP, "CGNS section 1 is not TRI_3 triangles");
    uint64_t ec;
    Data cd;
    if (!child(h, sections[0].addr, "ElementConnectivity", ec) || !node_data(h, ec, cd))
      h5fail(CF_EINVAL, "CGNS section without ElementConnectivity");
    const auto conn = as_int(cd, "ElementConnectivity");
    if ((int64_t)conn.size() < 3 * nelt) h5fail(CF_EINVAL, "CGNS connectivity shorter than the zone's element count");
    M.tri.resize(3 * (size_t)nelt);
    for (int64_t i = 0; i < 3 * nelt; ++i) {
      if (conn[i] < 1 || conn[i] > nnt) h5fail(CF_EINVAL, "CGNS element node id out of range");
      M.tri[i] = (int32_t)conn[i];
    }
    /* boundary conditions: inflow (BCInflow) and outflow (BCOutflow) node lists */
    M.ndinput.clear(); M.numero_ndinput.clear(); M.ndoutput.clear(); M.numero_ndoutput.clear();
    uint64_t zbc;
    if (child(h, zone, "ZoneBC", zbc)) {
      for (const Node& bc : children(h, zbc, "BC_t")) {
        Data td, pd;
        if (!node_data(h, bc.addr, td)) continue;
        const std::string type = trimmed(as_string(td));
        const bool in = type == "BCInflow", out = type == "BCOutflow";
        if (!in && !out) continue;
        uint64_t pl;
        if (!child(h, bc.addr, "PointList", pl) || !node_data(h, pl, pd)) continue;
        const auto nodes = as_int(pd, "PointList");
        if (nodes.size() <= 1) continue;
        const std::string name = trimmed(bc.name);
        int32_t number = 1;
        const auto& names = in ? inlet_names : outlet_names;
        for (size_t i = 0; i < names.size(); ++i)
          if (trimmed(names[i]) == name) number = (int32_t)(i + 1);
        auto& list = in ? M.ndinput : M.ndoutput;
        auto& nums = in ? M.numero_ndinput : M.numero_ndoutput;
        for (int64_t v : nodes) {
          if (v < 1 || v > nnt) h5fail(CF_EINVAL, "CGNS boundary node id out of range");
          list.push_back((int32_t)v);
          nums.push_back(number);
        }
      }
    }
    /* Manning per element */
    M.manning_elt.assign((size_t)nelt, 0.0);
    M.has_manning = false;
    uint64_t man;
    if (want_manning && child(h, zone, "Manning", man)) {
      const auto arrays = children(h, man, "DataArray_t");
      Data md;
      if (!arrays.empty() && node_data(h, arrays[0].addr, md)) {
        const auto v = as_double(md, "Manning");
        if ((int64_t)v.size() != nelt) h5fail(CF_EINVAL, "Manning does not have the zone's element count");
        M.manning_elt = v;
        M.has_manning = true;
      }
    }
    return CF_OK;
  } catch (const H5Error& e) {
    err = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    err = "host allocation failed reading " + path;
    return CF_ENOMEM;
  }
}

}  // namespace cf
