// Reader of the reference's k-space files (MRI_DATA::read_external_data,
// src/mri_data.cpp:769-906, written through src/hdf5_interface.cpp) without the HDF5
// library, which is not available to this build.  It implements the part of the HDF5 file
// format those files use, from the published format specification:
//   * superblock versions 0-3;
//   * groups as symbol tables (version-1 B-tree of group nodes, symbol table nodes, local
//     heap), or as link messages in the object header (compact new-style groups);
//   * object headers version 1 and 2, with continuation blocks;
//   * datasets with a dataspace, a datatype (little-endian integers, IEEE floats, and
//     compounds of two floats for complex values) and a contiguous or compact layout;
//   * scalar integer and float attributes (the "Kdata" group's Num_Encodings, Num_Coils,
//     trajectory_type*, dft_needed*).
// Chunked or filtered datasets, dense (fractal-heap) groups and big-endian data are
// rejected with MRG_ERR_UNSUPPORTED.  A damaged file gives MRG_ERR_INVALID: every read is
// bounded by its message or by the file's size, every allocation by the file's size, and
// continuation chains and B-tree walks are capped.  The file's data are read into the caller's host
// buffers, which may be pinned: mrg_h5_load_encode stages an encode through pinned memory
// into a plan (mrg_set_traj, mrg_set_data).
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "mrg_internal.h"

using namespace mrg;

namespace {

constexpr uint64_t kUndef = ~0ull;

struct H5Type {
  int cls = -1;        // 0 fixed-point, 1 floating point, 6 compound
  uint32_t size = 0;   // bytes per element
  bool is_signed = false;
  int ncomp = 0;       // compound: two members of one float type (complex)
  uint32_t comp_off[2] = {0, 0};
  uint32_t comp_size = 0;
};

struct H5Object {
  std::vector<uint64_t> dims;
  bool has_space = false;
  H5Type type;
  int layout = -1;  // 0 compact, 1 contiguous, 2 chunked
  uint64_t data_addr = kUndef, data_size = 0;
  std::vector<uint8_t> compact;
  bool filtered = false;
  uint64_t btree = kUndef, heap = kUndef;  // symbol-table group
  std::map<std::string, uint64_t> links;   // link-message group
  bool dense_links = false;
  struct Attr {
    H5Type type;
    std::vector<uint64_t> dims;
    std::vector<uint8_t> data;
  };
  std::map<std::string, Attr> attrs;
};

class H5File {
 public:
  ~H5File() {
    if (f_) std::fclose(f_);
  }
  mrg_status open(const char *path) {
    f_ = std::fopen(path, "rb");
    if (!f_) return fail(MRG_ERR_INVALID, std::string("cannot open ") + path);
    if (std::fseek(f_, 0, SEEK_END) != 0) return fail(MRG_ERR_INVALID, std::string("cannot seek in ") + path);
    const long end = std::ftell(f_);
    if (end < 0) return fail(MRG_ERR_INVALID, std::string("cannot size ") + path);
    fsize_ = (uint64_t)end;
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    for (uint64_t at = 0;; at = at ? 2 * at : 512) {  // the superblock sits at 0, 512, 1024, ...
      uint8_t b[8];
      if (!read_at(at, b, 8)) return fail(MRG_ERR_INVALID, "not an HDF5 file");
      if (!std::memcmp(b, sig, 8)) {
        sb_ = at;
        break;
      }
      if (at > (1ull << 30)) return fail(MRG_ERR_INVALID, "not an HDF5 file");
    }
    uint8_t v;
    read_at(sb_ + 8, &v, 1);
    if (v <= 1) {
      uint8_t h[16];
      if (!read_at(sb_ + 8, h, 16)) return fail(MRG_ERR_INVALID, "truncated superblock");
      so_ = h[5];
      sl_ = h[6];
      if (so_ != 8 || sl_ != 8) return fail(MRG_ERR_UNSUPPORTED, "HDF5 offsets/lengths other than 8 bytes");
      uint64_t p = sb_ + 8 + 16 + (v == 1 ? 4 : 0);
      base_ = rd_off(p);  // base address, then free-space, end of file and driver addresses
      p += 4 * so_;
      // root group symbol table entry: link name offset, object header address, cache type,
      // reserved, scratch pad (B-tree and local heap addresses when the cache type is 1)
      root_ = rd_off(p + so_);
      const uint32_t cache = (uint32_t)rd_le(p + 2 * so_, 4);
      if (cache == 1) {
        root_btree_ = rd_off(p + 2 * so_ + 8);
        root_heap_ = rd_off(p + 3 * so_ + 8);
      }
    } else if (v == 2 || v == 3) {
      uint8_t h[3];
      if (!read_at(sb_ + 9, h, 3)) return fail(MRG_ERR_INVALID, "truncated superblock");
      so_ = h[0];
      sl_ = h[1];
      if (so_ != 8 || sl_ != 8) return fail(MRG_ERR_UNSUPPORTED, "HDF5 offsets/lengths other than 8 bytes");
      const uint64_t p = sb_ + 12;  // base, superblock extension, end of file, root object header
      base_ = rd_off(p);
      root_ = rd_off(p + 3 * so_);
    } else {
      return fail(MRG_ERR_UNSUPPORTED, "HDF5 superblock version " + std::to_string(v));
    }
    return MRG_OK;
  }

  // Object at an absolute path ("/Kdata/KX_E0"; "Kdata/KX_E0" is the same).
  mrg_status find(const std::string &path, H5Object &out) {
    H5Object cur;
    MRG_TRY(load_object(root_, cur));
    if (cur.btree == kUndef && root_btree_ != kUndef) {
      cur.btree = root_btree_;
      cur.heap = root_heap_;
    }
    size_t i = 0;
    while (i < path.size()) {
      while (i < path.size() && path[i] == '/') i++;
      if (i >= path.size()) break;
      size_t j = path.find('/', i);
      if (j == std::string::npos) j = path.size();
      const std::string name = path.substr(i, j - i);
      uint64_t addr = kUndef;
      MRG_TRY(lookup(cur, name, &addr));
      if (addr == kUndef) return fail(MRG_ERR_INVALID, "HDF5 object not found: " + path);
      H5Object next;
      MRG_TRY(load_object(addr, next));
      cur = std::move(next);
      i = j;
    }
    out = std::move(cur);
    return MRG_OK;
  }

  // Raw element bytes of a dataset (contiguous or compact).
  mrg_status read_raw(const H5Object &o, uint8_t *dst, uint64_t nbytes) {
    if (o.filtered) return fail(MRG_ERR_UNSUPPORTED, "filtered (compressed) HDF5 datasets are not supported");
    if (o.layout == 0) {
      if (o.compact.size() < nbytes) return fail(MRG_ERR_INVALID, "compact dataset smaller than its dataspace");
      std::memcpy(dst, o.compact.data(), nbytes);
      return MRG_OK;
    }
    if (o.layout != 1) return fail(MRG_ERR_UNSUPPORTED, "chunked HDF5 datasets are not supported");
    if (o.data_addr == kUndef) {  // never written: the fill value, zero here
      std::memset(dst, 0, nbytes);
      return MRG_OK;
    }
    if (o.data_size < nbytes) return fail(MRG_ERR_INVALID, "contiguous dataset smaller than its dataspace");
    if (!fits(base_ + o.data_addr, nbytes) || !read_at(base_ + o.data_addr, dst, nbytes))
      return fail(MRG_ERR_INVALID, "truncated dataset");
    return MRG_OK;
  }

  // Elements and bytes of a dataset's dataspace, checked against where its data can be: the
  // compact bytes, the contiguous extent inside the file, or (never written) 64 GiB.
  mrg_status extent(const H5Object &o, uint64_t &count, uint64_t &bytes) const {
    count = 1;
    for (uint64_t d : o.dims) {
      if (d != 0 && count > (1ull << 48) / d) return fail(MRG_ERR_INVALID, "HDF5 dataspace too large");
      count *= d;
    }
    if (o.type.size == 0 || count > (1ull << 48) / o.type.size) return fail(MRG_ERR_INVALID, "HDF5 dataset too large");
    bytes = count * o.type.size;
    const uint64_t room = o.layout == 0 ? o.compact.size()
                          : o.data_addr == kUndef ? (1ull << 36)
                          : (o.data_size < fsize_ ? o.data_size : fsize_);
    if (bytes > room) return fail(MRG_ERR_INVALID, "HDF5 dataset larger than its storage");
    return MRG_OK;
  }

  static mrg_status fail(mrg_status s, const std::string &m) {
    set_error(m);
    return s;
  }

 private:
  FILE *f_ = nullptr;
  uint64_t fsize_ = 0, sb_ = 0, base_ = 0, root_ = kUndef, root_btree_ = kUndef, root_heap_ = kUndef;
  int so_ = 8, sl_ = 8;
  int visits_ = 0;  // B-tree nodes visited by the current lookup

  // [at, at + n) lies inside the file
  bool fits(uint64_t at, uint64_t n) const { return at <= fsize_ && n <= fsize_ - at; }
  bool read_at(uint64_t at, void *dst, size_t n) {
    if (!fits(at, n) || at > (uint64_t)0x7fffffffffffffffull) return false;
    if (std::fseek(f_, (long)at, SEEK_SET) != 0) return false;
    return std::fread(dst, 1, n, f_) == n;
  }
  uint64_t rd_le(uint64_t at, int n) {
    uint8_t b[8] = {0};
    if (n < 1 || n > 8 || !read_at(at, b, (size_t)n)) return kUndef;
    uint64_t v = 0;
    for (int k = n - 1; k >= 0; k--) v = (v << 8) | b[k];
    return v;
  }
  uint64_t rd_off(uint64_t at) { return rd_le(at, so_); }
  static uint64_t le(const uint8_t *p, int n) {
    uint64_t v = 0;
    for (int k = n - 1; k >= 0; k--) v = (v << 8) | p[k];
    return v;
  }

  mrg_status lookup(const H5Object &g, const std::string &name, uint64_t *addr) {
    auto it = g.links.find(name);
    if (it != g.links.end()) {
      *addr = it->second;
      return MRG_OK;
    }
    if (g.dense_links) return fail(MRG_ERR_UNSUPPORTED, "dense HDF5 link storage is not supported");
    if (g.btree == kUndef) return MRG_OK;
    std::vector<char> heap;
    MRG_TRY(load_heap(g.heap, heap));
    visits_ = 0;
    return search_btree(g.btree, heap, name, addr, 0);
  }

  mrg_status load_heap(uint64_t at, std::vector<char> &out) {
    uint8_t h[8];
    if (!read_at(base_ + at, h, 8) || std::memcmp(h, "HEAP", 4)) return fail(MRG_ERR_INVALID, "bad HDF5 local heap");
    const uint64_t size = rd_le(base_ + at + 8, sl_);
    const uint64_t data = rd_off(base_ + at + 8 + 2 * sl_);
    if (size > fsize_) return fail(MRG_ERR_INVALID, "bad HDF5 local heap size");
    out.assign(size + 1, 0);
    if (size && !read_at(base_ + data, out.data(), size)) return fail(MRG_ERR_INVALID, "truncated HDF5 local heap");
    return MRG_OK;
  }

  mrg_status search_btree(uint64_t at, const std::vector<char> &heap, const std::string &name, uint64_t *addr,
                          int depth) {
    if (depth > 32) return fail(MRG_ERR_INVALID, "HDF5 B-tree too deep");
    if (++visits_ > (1 << 16)) return fail(MRG_ERR_INVALID, "HDF5 B-tree too large");
    uint8_t h[8];
    if (!read_at(base_ + at, h, 8) || std::memcmp(h, "TREE", 4) || h[4] != 0)
      return fail(MRG_ERR_INVALID, "bad HDF5 group B-tree node");
    const int level = h[5];
    const int used = (int)le(h + 6, 2);
    uint64_t p = base_ + at + 8 + 2 * so_;  // after the siblings: key0, child0, key1, ...
    for (int k = 0; k < used; k++) {
      const uint64_t child = rd_off(p + sl_ + (uint64_t)k * (sl_ + so_));
      if (level > 0) {
        MRG_TRY(search_btree(child, heap, name, addr, depth + 1));
      } else {
        MRG_TRY(search_snod(child, heap, name, addr));
      }
      if (*addr != kUndef) return MRG_OK;
    }
    return MRG_OK;
  }

  mrg_status search_snod(uint64_t at, const std::vector<char> &heap, const std::string &name, uint64_t *addr) {
    uint8_t h[8];
    if (!read_at(base_ + at, h, 8) || std::memcmp(h, "SNOD", 4)) return fail(MRG_ERR_INVALID, "bad HDF5 symbol node");
    const int n = (int)le(h + 6, 2);
    const uint64_t esz = 2 * so_ + 4 + 4 + 16;
    for (int k = 0; k < n; k++) {
      const uint64_t e = base_ + at + 8 + k * esz;
      const uint64_t noff = rd_off(e);
      if (noff < heap.size() && name == std::string(heap.data() + noff)) {
        *addr = rd_off(e + so_);
        return MRG_OK;
      }
    }
    return MRG_OK;
  }

  // datatype message body -> H5Type
  mrg_status parse_type(const uint8_t *p, size_t n, H5Type &t) {
    if (n < 8) return fail(MRG_ERR_INVALID, "short HDF5 datatype");
    const int cls = p[0] & 15, ver = p[0] >> 4;
    t.cls = cls;
    t.size = (uint32_t)le(p + 4, 4);
    if (cls == 0) {
      if (p[1] & 1) return fail(MRG_ERR_UNSUPPORTED, "big-endian HDF5 data");
      if (t.size != 1 && t.size != 2 && t.size != 4 && t.size != 8)
        return fail(MRG_ERR_UNSUPPORTED, "HDF5 integer of size " + std::to_string(t.size));
      t.is_signed = (p[1] & 8) != 0;
    } else if (cls == 1) {
      if (p[1] & 1) return fail(MRG_ERR_UNSUPPORTED, "big-endian HDF5 data");
      if (t.size != 4 && t.size != 8) return fail(MRG_ERR_UNSUPPORTED, "HDF5 float of size " + std::to_string(t.size));
    } else if (cls == 6) {
      const int nm = (int)le(p + 1, 2);
      if (nm != 2) return fail(MRG_ERR_UNSUPPORTED, "HDF5 compound types other than (real, imag)");
      size_t q = 8;
      for (int m = 0; m < 2; m++) {
        size_t l = 0;
        while (q + l < n && p[q + l]) l++;
        size_t name_len = l + 1;
        if (ver < 3) name_len = (name_len + 7) & ~size_t(7);
        q += name_len;
        if (q + 4 > n) return fail(MRG_ERR_INVALID, "short HDF5 compound member");
        uint32_t off;
        if (ver < 3) {
          off = (uint32_t)le(p + q, 4);
          q += 4;
          if (ver == 1) q += 28;  // dimensionality, reserved, permutation, reserved, dimension sizes
        } else {
          int ob = t.size < 256 ? 1 : (t.size < 65536 ? 2 : 4);
          off = (uint32_t)le(p + q, ob);
          q += ob;
        }
        if (q + 8 > n) return fail(MRG_ERR_INVALID, "short HDF5 compound member");
        H5Type mt;
        MRG_TRY(parse_type(p + q, n - q, mt));
        if (mt.cls != 1) return fail(MRG_ERR_UNSUPPORTED, "HDF5 compound of non-float members");
        if ((uint64_t)off + mt.size > t.size) return fail(MRG_ERR_INVALID, "HDF5 compound member outside its element");
        if (m == 1 && mt.size != t.comp_size) return fail(MRG_ERR_UNSUPPORTED, "HDF5 compound of unequal members");
        t.comp_off[m] = off;
        t.comp_size = mt.size;
        q += 8 + 12;  // member header and floating-point properties
      }
      t.ncomp = 2;
    } else {
      return fail(MRG_ERR_UNSUPPORTED, "HDF5 datatype class " + std::to_string(cls));
    }
    return MRG_OK;
  }

  mrg_status parse_space(const uint8_t *p, size_t n, std::vector<uint64_t> &dims) {
    if (n < 8) return fail(MRG_ERR_INVALID, "short HDF5 dataspace");
    const int ver = p[0], rank = p[1];
    const size_t q = (ver == 1) ? 8 : 4;  // version 1: 4 reserved bytes; version 2: a type byte
    if ((ver != 1 && ver != 2) || q + (size_t)rank * sl_ > n) return fail(MRG_ERR_INVALID, "bad HDF5 dataspace");
    dims.clear();
    for (int d = 0; d < rank; d++) dims.push_back(le(p + q + (size_t)d * sl_, sl_));
    return MRG_OK;
  }

  mrg_status message(H5Object &o, int type, const uint8_t *p, size_t n, std::vector<std::pair<uint64_t, uint64_t>> &cont,
                     int ohver) {
    const auto shrt = [&]() { return fail(MRG_ERR_INVALID, "short HDF5 message " + std::to_string(type)); };
    switch (type) {
      case 0x0001:
        MRG_TRY(parse_space(p, n, o.dims));
        o.has_space = true;
        break;
      case 0x0003:
        MRG_TRY(parse_type(p, n, o.type));
        break;
      case 0x0008: {  // data layout
        if (n < 3) return shrt();
        const int ver = p[0];
        if (ver >= 3) {
          o.layout = p[1];
          if (o.layout == 0) {
            if (n < 4) return shrt();
            const size_t sz = (size_t)le(p + 2, 2);
            if (4 + sz > n) return shrt();
            o.compact.assign(p + 4, p + 4 + sz);
          } else if (o.layout == 1) {
            if (2 + (size_t)so_ + (size_t)sl_ > n) return shrt();
            o.data_addr = le(p + 2, so_);
            o.data_size = le(p + 2 + so_, sl_);
          }
        } else {
          const int rank = p[1];
          o.layout = p[2];
          if (o.layout == 1) {
            if (8 + (size_t)so_ + 4 * (size_t)rank > n) return shrt();
            o.data_addr = le(p + 8, so_);
            uint64_t sz = 1;  // bytes: the last of the sizes is the element size
            for (int d = 0; d < rank; d++) {
              const uint64_t e = le(p + 8 + so_ + 4 * d, 4);
              sz = (e != 0 && sz > (1ull << 48) / e) ? (1ull << 48) : sz * e;
            }
            o.data_size = sz;
          } else if (o.layout == 0) {
            const size_t q = 8 + 4 * (size_t)rank;
            if (q + 4 > n) return shrt();
            const size_t sz = (size_t)le(p + q, 4);
            if (q + 4 + sz > n) return shrt();
            o.compact.assign(p + q + 4, p + q + 4 + sz);
          }
        }
        if (o.data_addr == kUndef >> (64 - 8 * so_)) o.data_addr = kUndef;
        break;
      }
      case 0x000B:  // filter pipeline
        o.filtered = true;
        break;
      case 0x000C: {  // attribute
        if (n < 9) return shrt();
        const int ver = p[0];
        const size_t nl = (size_t)le(p + 2, 2), tl = (size_t)le(p + 4, 2), sl = (size_t)le(p + 6, 2);
        size_t q = (ver == 3) ? 9 : 8;
        auto pad = [&](size_t x) { return ver == 1 ? ((x + 7) & ~size_t(7)) : x; };
        if (q + pad(nl) > n) return shrt();
        std::string name(reinterpret_cast<const char *>(p + q), nl ? nl - 1 : 0);
        q += pad(nl);
        H5Object::Attr a;
        if (q + pad(tl) > n) return shrt();
        MRG_TRY(parse_type(p + q, tl, a.type));
        q += pad(tl);
        if (q + pad(sl) > n) return shrt();
        MRG_TRY(parse_space(p + q, sl, a.dims));
        q += pad(sl);
        if (q <= n) a.data.assign(p + q, p + n);
        o.attrs[name] = std::move(a);
        break;
      }
      case 0x0006: {  // link message (compact new-style group)
        if (n < 2) return shrt();
        const int flags = p[1];
        size_t q = 2;
        int ltype = 0;
        if (flags & 8) {
          if (q + 1 > n) return shrt();
          ltype = p[q++];
        }
        if (flags & 4) q += 8;  // creation order
        if (flags & 16) q += 1;  // character set
        const int lb = 1 << (flags & 3);
        if (q + lb > n) return shrt();
        const size_t nl = (size_t)le(p + q, lb);
        q += lb;
        if (nl > n || q + nl > n) return shrt();
        std::string name(reinterpret_cast<const char *>(p + q), nl);
        q += nl;
        if (ltype == 0) {  // hard link
          if (q + (size_t)so_ > n) return shrt();
          o.links[name] = le(p + q, so_);
        }
        break;
      }
      case 0x0002:  // link info: dense storage when the fractal heap address is defined
        if (n >= 2 + (size_t)so_) {
          size_t q = 2 + ((p[1] & 1) ? 8 : 0);
          if (q + (size_t)so_ > n) return shrt();
          if (le(p + q, so_) != (kUndef >> (64 - 8 * so_))) o.dense_links = true;
        }
        break;
      case 0x0010:  // continuation
        if ((size_t)so_ + (size_t)sl_ > n) return shrt();
        if (cont.size() >= 4096) return fail(MRG_ERR_INVALID, "too many HDF5 header continuations");
        cont.emplace_back(le(p, so_), le(p + so_, sl_));
        break;
      case 0x0011:  // symbol table
        if (2 * (size_t)so_ > n) return shrt();
        o.btree = le(p, so_);
        o.heap = le(p + so_, so_);
        break;
      default:
        break;
    }
    (void)ohver;
    return MRG_OK;
  }

  mrg_status load_object(uint64_t at, H5Object &o) {
    std::vector<std::pair<uint64_t, uint64_t>> cont;
    uint8_t h[16];
    if (!read_at(base_ + at, h, 16)) return fail(MRG_ERR_INVALID, "truncated HDF5 object header");
    if (!std::memcmp(h, "OHDR", 4)) {  // version 2
      const int flags = h[5];
      uint64_t p = base_ + at + 6;
      if (flags & 32) p += 16;  // times
      if (flags & 16) p += 4;   // attribute phase change values
      const int cb = 1 << (flags & 3);
      const uint64_t size0 = rd_le(p, cb);
      p += cb;
      MRG_TRY(walk_v2(o, p, size0, flags, cont));
      for (size_t k = 0; k < cont.size(); k++) {
        uint8_t s[4];
        const uint64_t ca = base_ + cont[k].first;
        if (!read_at(ca, s, 4) || std::memcmp(s, "OCHK", 4) || cont[k].second < 8)
          return fail(MRG_ERR_INVALID, "bad HDF5 continuation");
        MRG_TRY(walk_v2(o, ca + 4, cont[k].second - 8, flags, cont));
      }
      return MRG_OK;
    }
    if (h[0] != 1) return fail(MRG_ERR_UNSUPPORTED, "HDF5 object header version " + std::to_string(h[0]));
    const int nmsg = (int)le(h + 2, 2);
    const uint64_t size = le(h + 8, 4);
    int seen = 0;
    MRG_TRY(walk_v1(o, base_ + at + 16, size, nmsg, seen, cont));
    for (size_t k = 0; k < cont.size() && seen < nmsg; k++)
      MRG_TRY(walk_v1(o, base_ + cont[k].first, cont[k].second, nmsg, seen, cont));
    return MRG_OK;
  }

  mrg_status walk_v1(H5Object &o, uint64_t p, uint64_t size, int nmsg, int &seen,
                     std::vector<std::pair<uint64_t, uint64_t>> &cont) {
    if (!fits(p, size)) return fail(MRG_ERR_INVALID, "truncated HDF5 object header");
    std::vector<uint8_t> blk(size);
    if (size && !read_at(p, blk.data(), size)) return fail(MRG_ERR_INVALID, "truncated HDF5 object header");
    size_t q = 0;
    while (q + 8 <= size && seen < nmsg) {
      const int type = (int)le(&blk[q], 2);
      const size_t len = (size_t)le(&blk[q + 2], 2);
      if (q + 8 + len > size) return fail(MRG_ERR_INVALID, "HDF5 message beyond its header");
      MRG_TRY(message(o, type, &blk[q + 8], len, cont, 1));
      q += 8 + len;
      seen++;
    }
    return MRG_OK;
  }

  mrg_status walk_v2(H5Object &o, uint64_t p, uint64_t size, int flags,
                     std::vector<std::pair<uint64_t, uint64_t>> &cont) {
    if (!fits(p, size)) return fail(MRG_ERR_INVALID, "truncated HDF5 object header");
    std::vector<uint8_t> blk(size);
    if (size && !read_at(p, blk.data(), size)) return fail(MRG_ERR_INVALID, "truncated HDF5 object header");
    const size_t hdr = (flags & 4) ? 6 : 4;
    size_t q = 0;
    while (q + hdr <= size) {
      const int type = blk[q];
      const size_t len = (size_t)le(&blk[q + 1], 2);
      if (q + hdr + len > size) break;  // gap at the end of the block
      MRG_TRY(message(o, type, &blk[q + hdr], len, cont, 2));
      q += hdr + len;
    }
    return MRG_OK;
  }
};

// Elements of a dataspace
uint64_t count_of(const std::vector<uint64_t> &dims) {
  uint64_t n = 1;
  for (uint64_t d : dims) n *= d;
  return n;
}

// Converts n elements of type t to float (real) or float pairs (complex).
mrg_status convert(const H5Type &t, const uint8_t *src, uint64_t n, float *dst, bool complex_out) {
  for (uint64_t i = 0; i < n; i++) {
    const uint8_t *e = src + i * t.size;
    auto fl = [](const uint8_t *p, uint32_t sz) -> float {
      if (sz == 4) {
        float v;
        std::memcpy(&v, p, 4);
        return v;
      }
      double v;
      std::memcpy(&v, p, 8);
      return (float)v;
    };
    if (t.cls == 6) {
      if (!complex_out) return H5File::fail(MRG_ERR_INVALID, "complex dataset read as real");
      dst[2 * i] = fl(e + t.comp_off[0], t.comp_size);
      dst[2 * i + 1] = fl(e + t.comp_off[1], t.comp_size);
      continue;
    }
    float v = 0.f;
    if (t.cls == 1) {
      v = fl(e, t.size);
    } else {
      uint64_t u = 0;
      for (int k = (int)t.size - 1; k >= 0; k--) u = (u << 8) | e[k];
      if (t.is_signed && t.size < 8 && (u >> (8 * t.size - 1)) & 1) u |= ~0ull << (8 * t.size);
      v = t.is_signed ? (float)(int64_t)u : (float)u;
    }
    if (complex_out) {
      dst[2 * i] = v;
      dst[2 * i + 1] = 0.f;
    } else {
      dst[i] = v;
    }
  }
  return MRG_OK;
}

// Runs f; an allocation failure or other exception becomes a status, since nothing may
// throw across the C ABI.
template <class F>
mrg_status guarded(F &&f) {
  try {
    return f();
  } catch (const std::bad_alloc &) {
    set_error("out of host memory reading an HDF5 file");
    return MRG_ERR_NOMEM;
  } catch (const std::exception &e) {
    set_error(std::string("HDF5 reader: ") + e.what());
    return MRG_ERR_INVALID;
  }
}

}  // namespace

struct mrg_h5 {
  H5File file;
  float *pinned = nullptr;  // staging for mrg_h5_load_encode
  size_t pinned_bytes = 0;
  ~mrg_h5() {
    if (pinned) cudaFreeHost(pinned);
  }
};

extern "C" {

mrg_status mrg_h5_open(const char *path, mrg_h5 **out) {
  if (!path || !out) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  *out = nullptr;
  return guarded([&]() -> mrg_status {
    std::unique_ptr<mrg_h5> h(new mrg_h5());
    MRG_TRY(h->file.open(path));
    *out = h.release();
    return MRG_OK;
  });
}

mrg_status mrg_h5_close(mrg_h5 *h) {
  delete h;
  return MRG_OK;
}

mrg_status mrg_h5_attr_int(mrg_h5 *h, const char *group, const char *name, int *value) {
  if (!h || !group || !name || !value) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  return guarded([&]() -> mrg_status {
    H5Object g;
    MRG_TRY(h->file.find(group, g));
    auto it = g.attrs.find(name);
    if (it == g.attrs.end()) return H5File::fail(MRG_ERR_INVALID, std::string("attribute not found: ") + name);
    const H5Object::Attr &a = it->second;
    if (a.type.cls != 0 || a.type.size > 8 || a.data.size() < a.type.size || count_of(a.dims) != 1)
      return H5File::fail(MRG_ERR_INVALID, std::string("attribute is not a scalar integer: ") + name);
    float v;
    MRG_TRY(convert(a.type, a.data.data(), 1, &v, false));
    int64_t u = 0;
    for (int k = (int)a.type.size - 1; k >= 0; k--) u = (u << 8) | a.data[k];
    if (a.type.is_signed && a.type.size < 8 && ((uint64_t)u >> (8 * a.type.size - 1)) & 1)
      u = (int64_t)((uint64_t)u | (~0ull << (8 * a.type.size)));
    *value = (int)u;
    return MRG_OK;
  });
}

mrg_status mrg_h5_dataset_info(mrg_h5 *h, const char *path, int *rank, int64_t dims[8], int *is_complex) {
  if (!h || !path) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  return guarded([&]() -> mrg_status {
    H5Object o;
    MRG_TRY(h->file.find(path, o));
    if (!o.has_space || o.type.cls < 0) return H5File::fail(MRG_ERR_INVALID, std::string("not a dataset: ") + path);
    if (o.dims.size() > 8) return H5File::fail(MRG_ERR_UNSUPPORTED, "dataset rank above 8");
    uint64_t cnt = 0, bytes = 0;
    MRG_TRY(h->file.extent(o, cnt, bytes));  // dims that no storage in the file could hold are rejected
    if (rank) *rank = (int)o.dims.size();
    if (dims)
      for (size_t d = 0; d < o.dims.size(); d++) dims[d] = (int64_t)o.dims[d];
    if (is_complex) *is_complex = o.type.cls == 6;
    return MRG_OK;
  });
}

// Reads a whole dataset as float32 (real) or complex64 (complex = 1) into dst (n elements).
mrg_status mrg_h5_read(mrg_h5 *h, const char *path, int complex_out, void *dst, int64_t n) {
  if (!h || !path || !dst || n < 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  return guarded([&]() -> mrg_status {
    H5Object o;
    MRG_TRY(h->file.find(path, o));
    if (!o.has_space || o.type.cls < 0) return H5File::fail(MRG_ERR_INVALID, std::string("not a dataset: ") + path);
    uint64_t cnt = 0, bytes = 0;
    MRG_TRY(h->file.extent(o, cnt, bytes));
    if ((int64_t)cnt != n)
      return H5File::fail(MRG_ERR_INVALID, std::string("dataset ") + path + " holds " + std::to_string(cnt) +
                                               " elements, not " + std::to_string(n));
    std::vector<uint8_t> raw((size_t)bytes);
    MRG_TRY(h->file.read_raw(o, raw.data(), raw.size()));
    return convert(o.type, raw.data(), cnt, static_cast<float *>(dst), complex_out != 0);
  });
}

mrg_status mrg_h5_mri_info(mrg_h5 *h, int *num_encodings, int *num_coils, int64_t *samples, int max_encodings) {
  if (!h) {
    set_error("null argument");
    return MRG_ERR_INVALID;
  }
  int ne = 0, nc = 0;
  MRG_TRY(mrg_h5_attr_int(h, "Kdata", "Num_Encodings", &ne));
  MRG_TRY(mrg_h5_attr_int(h, "Kdata", "Num_Coils", &nc));
  if (num_encodings) *num_encodings = ne;
  if (num_coils) *num_coils = nc;
  for (int e = 0; samples && e < ne && e < max_encodings; e++) {
    int64_t dims[8];
    int rank = 0;
    MRG_TRY(mrg_h5_dataset_info(h, ("Kdata/KX_E" + std::to_string(e)).c_str(), &rank, dims, nullptr));
    int64_t m = 1;
    for (int d = 0; d < rank; d++) m *= dims[d];
    samples[e] = m;
  }
  return MRG_OK;
}

mrg_status mrg_h5_load_encode(mrg_h5 *h, int encode, mrg_plan *plan, int frame, void *stream) {
  if (!h || !plan || encode < 0) {
    set_error("bad argument");
    return MRG_ERR_INVALID;
  }
  int ne = 0, nc = 0;
  MRG_TRY(mrg_h5_attr_int(h, "Kdata", "Num_Encodings", &ne));
  MRG_TRY(mrg_h5_attr_int(h, "Kdata", "Num_Coils", &nc));
  if (encode >= ne) return H5File::fail(MRG_ERR_INVALID, "encode beyond Num_Encodings");
  if (nc < 1 || nc > 4096) return H5File::fail(MRG_ERR_INVALID, "Num_Coils out of range: " + std::to_string(nc));
  int64_t M = 0;
  {
    int64_t dims[8];
    int rank = 0;
    MRG_TRY(mrg_h5_dataset_info(h, ("Kdata/KX_E" + std::to_string(encode)).c_str(), &rank, dims, nullptr));
    M = 1;
    for (int d = 0; d < rank; d++) M *= dims[d];
  }
  // pinned staging: kx, ky, kz, kw, then nc coils of complex samples (M is bounded by the
  // file's size through mrg_h5_dataset_info)
  if (M < 1 || (uint64_t)M > (1ull << 40)) return H5File::fail(MRG_ERR_INVALID, "bad sample count");
  const size_t need = sizeof(float) * (size_t)M * (4 + 2 * (size_t)nc);
  if (h->pinned_bytes < need) {
    if (h->pinned) cudaFreeHost(h->pinned);
    h->pinned = nullptr;
    h->pinned_bytes = 0;
    MRG_CUDA(cudaMallocHost(&h->pinned, need));
    h->pinned_bytes = need;
  }
  float *k[4];
  const char *names[4] = {"KX_E", "KY_E", "KZ_E", "KW_E"};
  for (int a = 0; a < 4; a++) {
    k[a] = h->pinned + (size_t)a * M;
    MRG_TRY(mrg_h5_read(h, ("Kdata/" + std::string(names[a]) + std::to_string(encode)).c_str(), 0, k[a], M));
  }
  float *d = h->pinned + 4 * (size_t)M;
  for (int c = 0; c < nc; c++)
    MRG_TRY(mrg_h5_read(h, ("Kdata/KData_E" + std::to_string(encode) + "_C" + std::to_string(c)).c_str(), 1,
                        d + 2 * (size_t)c * M, M));
  MRG_TRY(mrg_set_traj(plan, frame, k[0], k[1], k[2], k[3], M, stream));
  return mrg_set_data(plan, frame, d, M, stream);
}

}  // extern "C"
