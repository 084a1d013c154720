/* Writer of HDF5 files holding one-dimensional datasets in the root group.
 *
 * Every file sledgehamr writes (level data, slices, spectra, projections,
 * gravitational-wave spectra) is a flat set of 1-D datasets created with
 * utils::hdf5::Write (source/utils/hdf5_utils.h:80-104): IEEE float data,
 * little endian (ints are stored as 64-bit floats, hdf5_utils.h:93-95),
 * default dataset properties, in a file made by H5Fcreate with default
 * properties.  No HDF5 library is linked here; this writer lays out the
 * same structures the library's default (earliest) file format uses, from
 * the published HDF5 file format specification:
 *
 *   superblock version 0 (8-byte offsets and lengths, group leaf K 4,
 *   internal K 16) whose root symbol-table entry caches the root group's
 *   B-tree and local heap;
 *   the root group: a version-1 object header with one symbol-table
 *   message, a version-1 B-tree of type 0 over symbol-table nodes (SNOD,
 *   up to 2 * leaf K entries each, names in strcmp order), and a local heap
 *   holding the names (offset 0 is the empty string, each name NUL-padded
 *   to a multiple of 8 bytes, no free block);
 *   per dataset a version-1 object header of 256 message bytes with a
 *   dataspace (version 1, rank 1, maximum dimension = dimension), a
 *   datatype (IEEE F32LE or F64LE), a version-2 fill-value message, a
 *   version-3 contiguous layout message and a NIL message as padding, and
 *   the raw data after all metadata.
 *
 * These are the structures and message versions found in the reference's
 * own data file data/spectra_ks.hdf5 (written by h5py); the tests read both
 * that file and this writer's output with one parser of the specification.
 * Host only, free of CUDA.
 */
#ifndef SH_HDF5_H_
#define SH_HDF5_H_

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace sh {
namespace h5 {

constexpr uint64_t kUndef = ~0ull;
constexpr int kLeafK = 4;       /* symbol-table node holds 2K entries */
constexpr int kInternalK = 16;  /* group B-tree node holds 2K children */
constexpr int kSuperblockBytes = 96;
constexpr int kRootHeaderBytes = 16 + 8 + 16;
constexpr int kBtreeNodeBytes = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
constexpr int kHeapHeaderBytes = 32;
constexpr int kSnodBytes = 8 + 2 * kLeafK * 40;
constexpr int kDatasetMessageBytes = 256;
constexpr int kDatasetHeaderBytes = 16 + kDatasetMessageBytes;

enum Type { kF32 = 4, kF64 = 8 };

struct Dataset {
    int type = kF64;
    uint64_t n = 0;
    std::vector<unsigned char> bytes;
};

/* Little-endian byte image under construction. */
class Image {
  public:
    explicit Image(size_t n) : b_(n, 0) {}
    void u8(size_t at, unsigned v) { b_[at] = (unsigned char)v; }
    void u16(size_t at, unsigned v) { put(at, v, 2); }
    void u32(size_t at, uint64_t v) { put(at, v, 4); }
    void u64(size_t at, uint64_t v) { put(at, v, 8); }
    void bytes(size_t at, const void *p, size_t n) { std::memcpy(&b_[at], p, n); }
    const std::vector<unsigned char> &data() const { return b_; }

  private:
    void put(size_t at, uint64_t v, int n) {
        for (int q = 0; q < n; ++q) b_[at + q] = (unsigned char)(v >> (8 * q));
    }
    std::vector<unsigned char> b_;
};

inline bool little_endian_host() {
    const uint16_t one = 1;
    unsigned char c;
    std::memcpy(&c, &one, 1);
    return c == 1;
}

/* A name HDF5 accepts as one link of the root group. */
inline bool valid_name(const std::string &s) {
    return !s.empty() && s != "." && s.find('/') == std::string::npos &&
           s.find('\0') == std::string::npos;
}

class Writer {
  public:
    /* Adds a dataset of n values; false (with a message) for an invalid or
     * repeated name. */
    bool add_f64(const std::string &name, const double *v, uint64_t n, std::string *err) {
        return add(name, kF64, v, n, err);
    }
    bool add_f32(const std::string &name, const float *v, uint64_t n, std::string *err) {
        return add(name, kF32, v, n, err);
    }
    /* Integers are stored as F64LE, as utils::hdf5::Write does. */
    template <typename I>
    bool add_int_as_f64(const std::string &name, const I *v, uint64_t n, std::string *err) {
        std::vector<double> d(n);
        for (uint64_t q = 0; q < n; ++q) d[q] = (double)v[q];
        return add(name, kF64, d.data(), n, err);
    }
    /* Takes the bytes of n values of `type` without copying. */
    bool add_bytes(const std::string &name, int type, std::vector<unsigned char> &&bytes,
                   uint64_t n, std::string *err) {
        if (!check(name, type, err)) return false;
        if (bytes.size() != n * (uint64_t)type) {
            if (err) *err = "dataset " + name + ": byte count does not match its length";
            return false;
        }
        Dataset &d = sets_[name];
        d.type = type;
        d.n = n;
        d.bytes = std::move(bytes);
        return true;
    }
    size_t size() const { return sets_.size(); }
    bool contains(const std::string &name) const { return sets_.count(name) != 0; }

    /* Metadata of the file (everything before the raw data) and the offset
     * of each dataset's data, in name order. */
    std::vector<unsigned char> metadata(std::vector<uint64_t> *data_at, uint64_t *eof) const;

    /* Writes the file; false with a message on an I/O error. */
    bool write(const std::string &path, std::string *err) const {
        if (!little_endian_host()) {
            if (err) *err = "HDF5 writer: big-endian host";
            return false;
        }
        std::vector<uint64_t> at;
        uint64_t eof = 0;
        const std::vector<unsigned char> meta = metadata(&at, &eof);
        FILE *f = std::fopen(path.c_str(), "wb");
        if (!f) {
            if (err) *err = "cannot create " + path;
            return false;
        }
        bool ok = std::fwrite(meta.data(), 1, meta.size(), f) == meta.size();
        for (const auto &kv : sets_)
            if (ok && !kv.second.bytes.empty())
                ok = std::fwrite(kv.second.bytes.data(), 1, kv.second.bytes.size(), f) ==
                     kv.second.bytes.size();
        ok = (std::fclose(f) == 0) && ok;
        if (!ok && err) *err = "write to " + path + " failed";
        return ok;
    }

  private:
    bool check(const std::string &name, int type, std::string *err) const {
        if (!valid_name(name)) {
            if (err) *err = "invalid dataset name '" + name + "'";
            return false;
        }
        if (type != kF32 && type != kF64) {
            if (err) *err = "dataset " + name + ": type must be F32 or F64";
            return false;
        }
        if (sets_.count(name)) {
            if (err) *err = "dataset " + name + " already exists";
            return false;
        }
        return true;
    }
    bool add(const std::string &name, int type, const void *v, uint64_t n, std::string *err) {
        if (!check(name, type, err)) return false;
        if (n && !v) {
            if (err) *err = "dataset " + name + ": no data";
            return false;
        }
        std::vector<unsigned char> b(n * (uint64_t)type);
        if (n) std::memcpy(b.data(), v, b.size());
        return add_bytes(name, type, std::move(b), n, err);
    }

    /* std::string orders like strcmp (unsigned bytes), the order of HDF5's
     * group B-tree */
    std::map<std::string, Dataset> sets_;
};

inline std::vector<unsigned char> Writer::metadata(std::vector<uint64_t> *data_at,
                                                   uint64_t *eof) const {
    const size_t n = sets_.size();
    std::vector<const std::string *> names;
    std::vector<const Dataset *> sets;
    for (const auto &kv : sets_) {
        names.push_back(&kv.first);
        sets.push_back(&kv.second);
    }

    /* symbol-table nodes: consecutive runs of at most 2 * leaf K names */
    const size_t per_snod = 2 * kLeafK;
    const size_t nsnod = (n + per_snod - 1) / per_snod;

    /* B-tree levels, bottom up: level 0 points at the SNODs, each higher
     * level at the nodes below, at most 2 * internal K children per node */
    const size_t fan = 2 * kInternalK;
    std::vector<size_t> level_nodes;
    {
        size_t c = nsnod;
        do {
            const size_t nodes = c == 0 ? 1 : (c + fan - 1) / fan;
            level_nodes.push_back(nodes);
            c = nodes;
        } while (c > 1);
    }
    size_t nbtree = 0;
    for (size_t v : level_nodes) nbtree += v;

    /* local heap data: "" at 0, then each name NUL-padded to 8 bytes */
    std::vector<uint64_t> name_off(n);
    uint64_t heap_size = 8;
    for (size_t q = 0; q < n; ++q) {
        name_off[q] = heap_size;
        heap_size += (names[q]->size() + 1 + 7) / 8 * 8;
    }

    /* addresses */
    const uint64_t root_hdr = kSuperblockBytes;
    const uint64_t btree0 = root_hdr + kRootHeaderBytes;
    const uint64_t heap_hdr = btree0 + (uint64_t)nbtree * kBtreeNodeBytes;
    const uint64_t heap_data = heap_hdr + kHeapHeaderBytes;
    const uint64_t snod0 = heap_data + heap_size;
    const uint64_t dhdr0 = snod0 + (uint64_t)nsnod * kSnodBytes;
    const uint64_t meta_end = dhdr0 + (uint64_t)n * kDatasetHeaderBytes;
    std::vector<uint64_t> at(n);
    uint64_t end = meta_end;
    for (size_t q = 0; q < n; ++q) {
        at[q] = sets[q]->n ? end : kUndef;
        end += sets[q]->bytes.size();
    }

    /* node addresses per level; level L node j at btree0 + (offset of level
     * L, counted from the root down) so that the root is the first node */
    std::vector<uint64_t> level_base(level_nodes.size());
    {
        uint64_t a = btree0;
        for (size_t L = level_nodes.size(); L-- > 0;) {
            level_base[L] = a;
            a += (uint64_t)level_nodes[L] * kBtreeNodeBytes;
        }
    }
    const uint64_t root_btree = level_base.back();

    Image im((size_t)meta_end);

    /* superblock version 0 */
    static const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    im.bytes(0, sig, 8);
    im.u8(13, 8); /* size of offsets */
    im.u8(14, 8); /* size of lengths */
    im.u16(16, kLeafK);
    im.u16(18, kInternalK);
    im.u64(24, 0);      /* base address */
    im.u64(32, kUndef); /* free-space info */
    im.u64(40, end);    /* end of file */
    im.u64(48, kUndef); /* driver info */
    /* root symbol-table entry, scratch pad caching the B-tree and heap */
    im.u64(56, 0);
    im.u64(64, root_hdr);
    im.u32(72, 1);
    im.u64(80, root_btree);
    im.u64(88, heap_hdr);

    /* root group object header: one symbol-table message */
    im.u8(root_hdr, 1);
    im.u16(root_hdr + 2, 1);
    im.u32(root_hdr + 4, 1);
    im.u32(root_hdr + 8, 24);
    im.u16(root_hdr + 16, 0x11);
    im.u16(root_hdr + 18, 16);
    im.u64(root_hdr + 24, root_btree);
    im.u64(root_hdr + 32, heap_hdr);

    /* largest name of each SNOD, then of each node per level */
    std::vector<uint64_t> child_max(nsnod);
    for (size_t s = 0; s < nsnod; ++s) {
        const size_t last = std::min(n, (s + 1) * per_snod) - 1;
        child_max[s] = name_off[last];
    }
    uint64_t left_key = 0;
    for (size_t L = 0; L < level_nodes.size(); ++L) {
        const size_t nchild = L == 0 ? nsnod : level_nodes[L - 1];
        std::vector<uint64_t> node_max(level_nodes[L], 0);
        left_key = 0;
        for (size_t j = 0; j < level_nodes[L]; ++j) {
            const uint64_t a = level_base[L] + (uint64_t)j * kBtreeNodeBytes;
            const size_t c0 = j * fan;
            const size_t c1 = std::min(nchild, c0 + fan);
            im.bytes(a, "TREE", 4);
            im.u8(a + 4, 0); /* group node */
            im.u8(a + 5, (unsigned)L);
            im.u16(a + 6, (unsigned)(c1 - c0));
            im.u64(a + 8, j > 0 ? a - kBtreeNodeBytes : kUndef);
            im.u64(a + 16, j + 1 < level_nodes[L] ? a + kBtreeNodeBytes : kUndef);
            uint64_t p = a + 24;
            im.u64(p, left_key);
            for (size_t c = c0; c < c1; ++c) {
                const uint64_t child = L == 0 ? snod0 + (uint64_t)c * kSnodBytes
                                              : level_base[L - 1] + (uint64_t)c * kBtreeNodeBytes;
                im.u64(p + 8, child);
                im.u64(p + 16, child_max[c]);
                p += 16;
            }
            if (c1 > c0) left_key = child_max[c1 - 1];
            node_max[j] = left_key;
        }
        child_max = node_max;
    }

    /* local heap */
    im.bytes(heap_hdr, "HEAP", 4);
    im.u64(heap_hdr + 8, heap_size);
    im.u64(heap_hdr + 16, 1); /* no free block */
    im.u64(heap_hdr + 24, heap_data);
    for (size_t q = 0; q < n; ++q) im.bytes(heap_data + name_off[q], names[q]->data(), names[q]->size());

    /* symbol-table nodes */
    for (size_t s = 0; s < nsnod; ++s) {
        const uint64_t a = snod0 + (uint64_t)s * kSnodBytes;
        const size_t q0 = s * per_snod, q1 = std::min(n, q0 + per_snod);
        im.bytes(a, "SNOD", 4);
        im.u8(a + 4, 1);
        im.u16(a + 6, (unsigned)(q1 - q0));
        for (size_t q = q0; q < q1; ++q) {
            const uint64_t e = a + 8 + 40 * (q - q0);
            im.u64(e, name_off[q]);
            im.u64(e + 8, dhdr0 + (uint64_t)q * kDatasetHeaderBytes);
        }
    }

    /* dataset object headers */
    for (size_t q = 0; q < n; ++q) {
        const Dataset &d = *sets[q];
        const uint64_t h = dhdr0 + (uint64_t)q * kDatasetHeaderBytes;
        im.u8(h, 1);
        im.u16(h + 2, 5);
        im.u32(h + 4, 1);
        im.u32(h + 8, kDatasetMessageBytes);
        uint64_t m = h + 16;
        /* dataspace, version 1: rank 1 with maximum dimensions */
        im.u16(m, 0x01);
        im.u16(m + 2, 24);
        im.u8(m + 8, 1);
        im.u8(m + 9, 1);
        im.u8(m + 10, 1);
        im.u64(m + 16, d.n);
        im.u64(m + 24, d.n);
        m += 32;
        /* datatype: IEEE little-endian float, constant */
        im.u16(m, 0x03);
        im.u16(m + 2, 24);
        im.u8(m + 4, 1);
        im.u8(m + 8, 0x11);                  /* version 1, floating point */
        im.u8(m + 9, 0x20);                  /* implied mantissa msb */
        im.u8(m + 10, d.type == kF64 ? 63 : 31); /* sign bit */
        im.u32(m + 12, (uint64_t)d.type);
        im.u16(m + 16, 0);                   /* bit offset */
        im.u16(m + 18, d.type == kF64 ? 64 : 32);
        im.u8(m + 20, d.type == kF64 ? 52 : 23); /* exponent location */
        im.u8(m + 21, d.type == kF64 ? 11 : 8);
        im.u8(m + 22, 0);                        /* mantissa location */
        im.u8(m + 23, d.type == kF64 ? 52 : 23);
        im.u32(m + 24, d.type == kF64 ? 1023 : 127);
        m += 32;
        /* fill value, version 2: late allocation, written if set, defined
         * with the default (zero-length) value */
        im.u16(m, 0x05);
        im.u16(m + 2, 8);
        im.u8(m + 4, 1);
        im.u8(m + 8, 2);
        im.u8(m + 9, 2);
        im.u8(m + 10, 2);
        im.u8(m + 11, 1);
        m += 16;
        /* layout, version 3: contiguous */
        im.u16(m, 0x08);
        im.u16(m + 2, 24);
        im.u8(m + 8, 3);
        im.u8(m + 9, 1);
        im.u64(m + 10, at[q]);
        im.u64(m + 18, d.bytes.size());
        m += 32;
        /* NIL message up to the header's message bytes */
        im.u16(m, 0x00);
        im.u16(m + 2, (unsigned)(h + 16 + kDatasetMessageBytes - m - 8));
    }

    if (data_at) *data_at = at;
    if (eof) *eof = end;
    return im.data();
}

/* Reader of the files this writer produces (the structures listed at the
 * top: superblock version 0, a root group of version-1 B-tree nodes over
 * symbol-table nodes with a local heap of names, version-1 object headers
 * with dataspace, datatype and contiguous layout messages): every 1-D
 * F32LE or F64LE dataset of the root group, by name.  Other structures are
 * rejected with a message.  Used to restart from checkpoint headers. */
class Reader {
  public:
    bool open(const std::string &path, std::string *err) {
        FILE *f = std::fopen(path.c_str(), "rb");
        if (!f) return fail(err, "cannot open " + path);
        std::fseek(f, 0, SEEK_END);
        const long n = std::ftell(f);
        std::fseek(f, 0, SEEK_SET);
        buf_.assign(n > 0 ? (size_t)n : 0, 0);
        const bool ok = n > 0 && std::fread(buf_.data(), 1, buf_.size(), f) == buf_.size();
        std::fclose(f);
        if (!ok) return fail(err, "cannot read " + path);
        static const unsigned char sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
        if (buf_.size() < kSuperblockBytes || std::memcmp(buf_.data(), sig, 8) != 0 ||
            buf_[8] != 0 || buf_[13] != 8 || buf_[14] != 8)
            return fail(err, path + ": not an HDF5 file with a version-0 superblock");
        uint64_t btree = 0, heap = 0;
        if (!u64(80, &btree) || !u64(88, &heap)) return fail(err, path + ": truncated");
        uint64_t heap_data = 0;
        if (!has(heap, 32) || std::memcmp(&buf_[heap], "HEAP", 4) != 0 ||
            !u64(heap + 24, &heap_data))
            return fail(err, path + ": no local heap of the root group");
        heap_data_ = heap_data;
        sets_.clear();
        if (!walk(btree, 0, err)) return false;
        return true;
    }
    bool has_dataset(const std::string &name) const { return sets_.count(name) != 0; }
    /* values of dataset `name` as FP64 (F32 data widened) */
    bool get(const std::string &name, std::vector<double> *out, std::string *err) const {
        auto it = sets_.find(name);
        if (it == sets_.end()) return fail(err, "no dataset " + name);
        const Entry &e = it->second;
        out->resize(e.n);
        if (e.n == 0) return true;
        if (!has(e.addr, e.n * (uint64_t)e.type)) return fail(err, name + ": data out of file");
        for (uint64_t q = 0; q < e.n; ++q) {
            if (e.type == kF64) {
                double v;
                std::memcpy(&v, &buf_[e.addr + 8 * q], 8);
                (*out)[q] = v;
            } else {
                float v;
                std::memcpy(&v, &buf_[e.addr + 4 * q], 4);
                (*out)[q] = v;
            }
        }
        return true;
    }

  private:
    struct Entry {
        int type = kF64;
        uint64_t n = 0, addr = 0;
    };
    static bool fail(std::string *err, const std::string &m) {
        if (err) *err = m;
        return false;
    }
    bool has(uint64_t at, uint64_t n) const { return at <= buf_.size() && n <= buf_.size() - at; }
    bool u64(uint64_t at, uint64_t *v) const {
        if (!has(at, 8)) return false;
        uint64_t x = 0;
        for (int q = 7; q >= 0; --q) x = (x << 8) | buf_[at + q];
        *v = x;
        return true;
    }
    uint64_t un(uint64_t at, int n) const {
        uint64_t x = 0;
        for (int q = n - 1; q >= 0; --q) x = (x << 8) | buf_[at + q];
        return x;
    }
    bool walk(uint64_t node, int depth, std::string *err) {
        if (depth > 16 || !has(node, 24)) return fail(err, "bad group B-tree node");
        if (std::memcmp(&buf_[node], "TREE", 4) == 0) {
            if (buf_[node + 4] != 0) return fail(err, "not a group B-tree");
            const unsigned used = (unsigned)un(node + 6, 2);
            for (unsigned c = 0; c < used; ++c) {
                uint64_t child = 0;
                if (!u64(node + 24 + 8 + 16 * c, &child)) return fail(err, "truncated B-tree");
                if (!walk(child, depth + 1, err)) return false;
            }
            return true;
        }
        if (std::memcmp(&buf_[node], "SNOD", 4) == 0) {
            const unsigned n = (unsigned)un(node + 6, 2);
            for (unsigned q = 0; q < n; ++q) {
                const uint64_t e = node + 8 + 40 * q;
                uint64_t name_off = 0, hdr = 0;
                if (!u64(e, &name_off) || !u64(e + 8, &hdr)) return fail(err, "truncated SNOD");
                const uint64_t at = heap_data_ + name_off;
                std::string name;
                while (has(at + name.size(), 1) && buf_[at + name.size()] != 0)
                    name.push_back((char)buf_[at + name.size()]);
                if (!dataset(name, hdr, err)) return false;
            }
            return true;
        }
        return fail(err, "unknown group node");
    }
    bool dataset(const std::string &name, uint64_t h, std::string *err) {
        if (!has(h, 16) || buf_[h] != 1) return fail(err, name + ": not a version-1 object header");
        const unsigned nmsg = (unsigned)un(h + 2, 2);
        const uint64_t size = un(h + 8, 4);
        uint64_t m = h + 16;
        const uint64_t end = h + 16 + size;
        if (!has(h + 16, size)) return fail(err, name + ": truncated object header");
        Entry e;
        bool space = false, type = false, layout = false;
        for (unsigned q = 0; q < nmsg && m + 8 <= end; ++q) {
            const unsigned mt = (unsigned)un(m, 2), ms = (unsigned)un(m + 2, 2);
            const uint64_t d = m + 8;
            if (mt == 0x01) { /* dataspace */
                const unsigned ver = buf_[d], rank = buf_[d + 1];
                if (rank != 1) return fail(err, name + ": not one-dimensional");
                e.n = un(d + (ver == 1 ? 8 : 4), 8);
                space = true;
            } else if (mt == 0x03) { /* datatype */
                if ((buf_[d] & 0x0F) != 1) return fail(err, name + ": not a floating-point type");
                const uint64_t sz = un(d + 4, 4);
                if (sz != 4 && sz != 8) return fail(err, name + ": float size");
                if (buf_[d + 1] & 1) return fail(err, name + ": big-endian data");
                e.type = (int)sz;
                type = true;
            } else if (mt == 0x08) { /* data layout */
                if (buf_[d] != 3 || buf_[d + 1] != 1)
                    return fail(err, name + ": not a version-3 contiguous layout");
                e.addr = un(d + 2, 8);
                layout = true;
            }
            m = d + ms;
        }
        if (!space || !type || !layout) return fail(err, name + ": incomplete dataset header");
        if (e.n == 0) e.addr = 0;
        sets_[name] = e;
        return true;
    }
    std::vector<unsigned char> buf_;
    uint64_t heap_data_ = 0;
    std::map<std::string, Entry> sets_;
};

} // namespace h5
} // namespace sh

#endif // SH_HDF5_H_
