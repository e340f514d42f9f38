// HDF5 subset reader/writer and material folders (see phmc_hdf5.h).
#include "phmc_hdf5.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <limits>
#include <sstream>
#include <stdexcept>

namespace phmc {
namespace {

// ------------------------------------------------------------- inflate
// RFC 1951 decoder: stored, fixed-Huffman and dynamic-Huffman blocks, with
// canonical Huffman codes decoded one bit at a time (counts per length, then
// symbols in code order).
class Inflate {
public:
    Inflate(const uint8_t* in, size_t n, std::vector<uint8_t>& out) : in_(in), n_(n), out_(out) {}

    void run() {
        bool last = false;
        while (!last) {
            last = bits(1) != 0;
            const int type = bits(2);
            if (type == 0) stored();
            else if (type == 1) fixed();
            else if (type == 2) dynamic();
            else fail("invalid block type");
        }
    }

private:
    struct Code {
        uint16_t count[16];
        uint16_t symbol[320];
    };
    const uint8_t* in_;
    size_t n_, pos_ = 0;
    uint32_t buf_ = 0;
    int cnt_ = 0;
    std::vector<uint8_t>& out_;

    [[noreturn]] static void fail(const char* what) { throw std::runtime_error(std::string("HDF5: deflate data: ") + what); }

    int bits(int need) {
        uint32_t v = buf_;
        while (cnt_ < need) {
            if (pos_ >= n_) fail("input ends early");
            v |= static_cast<uint32_t>(in_[pos_++]) << cnt_;
            cnt_ += 8;
        }
        buf_ = v >> need;
        cnt_ -= need;
        return static_cast<int>(v & ((1u << need) - 1u));
    }

    void stored() {
        buf_ = 0;
        cnt_ = 0; // to the byte boundary
        if (pos_ + 4 > n_) fail("stored block header");
        const unsigned len = in_[pos_] | (in_[pos_ + 1] << 8);
        const unsigned nlen = in_[pos_ + 2] | (in_[pos_ + 3] << 8);
        pos_ += 4;
        if (len != (~nlen & 0xffffu)) fail("stored length check");
        if (pos_ + len > n_) fail("stored block data");
        out_.insert(out_.end(), in_ + pos_, in_ + pos_ + len);
        pos_ += len;
    }

    static void build(Code& h, const uint8_t* length, int n) {
        std::fill(std::begin(h.count), std::end(h.count), 0);
        for (int s = 0; s < n; ++s) h.count[length[s]]++;
        if (h.count[0] == n) return; // no codes
        int left = 1;
        for (int len = 1; len < 16; ++len) {
            left <<= 1;
            left -= h.count[len];
            if (left < 0) fail("over-subscribed code");
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; ++len) offs[len + 1] = static_cast<uint16_t>(offs[len] + h.count[len]);
        for (int s = 0; s < n; ++s)
            if (length[s] != 0) h.symbol[offs[length[s]]++] = static_cast<uint16_t>(s);
    }

    int decode(const Code& h) {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= bits(1);
            const int count = h.count[len];
            if (code - count < first) return h.symbol[index + (code - first)];
            index += count;
            first += count;
            first <<= 1;
            code <<= 1;
        }
        fail("invalid code");
    }

    void codes(const Code& lencode, const Code& distcode) {
        static const uint16_t lbase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                                           35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
        static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
        static const uint16_t dbase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                           193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
        static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
        for (;;) {
            int sym = decode(lencode);
            if (sym < 256) {
                out_.push_back(static_cast<uint8_t>(sym));
            } else if (sym == 256) {
                return;
            } else {
                sym -= 257;
                if (sym >= 29) fail("invalid length symbol");
                const int len = lbase[sym] + bits(lext[sym]);
                const int ds = decode(distcode);
                if (ds >= 30) fail("invalid distance symbol");
                const size_t dist = dbase[ds] + bits(dext[ds]);
                if (dist > out_.size()) fail("distance before the output start");
                const size_t from = out_.size() - dist;
                for (int k = 0; k < len; ++k) out_.push_back(out_[from + k]);
            }
        }
    }

    void fixed() {
        static Code lc, dc;
        static bool ready = false;
        if (!ready) {
            uint8_t l[288];
            int s = 0;
            for (; s < 144; ++s) l[s] = 8;
            for (; s < 256; ++s) l[s] = 9;
            for (; s < 280; ++s) l[s] = 7;
            for (; s < 288; ++s) l[s] = 8;
            build(lc, l, 288);
            uint8_t d[30];
            std::fill(d, d + 30, 5);
            build(dc, d, 30);
            ready = true;
        }
        codes(lc, dc);
    }

    void dynamic() {
        static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
        const int nlen = bits(5) + 257, ndist = bits(5) + 1, ncode = bits(4) + 4;
        if (nlen > 286 || ndist > 30) fail("bad code counts");
        uint8_t lengths[320] = {0};
        for (int k = 0; k < ncode; ++k) lengths[order[k]] = static_cast<uint8_t>(bits(3));
        Code lc, dc;
        build(lc, lengths, 19);
        int idx = 0;
        while (idx < nlen + ndist) {
            int sym = decode(lc);
            if (sym < 16) {
                lengths[idx++] = static_cast<uint8_t>(sym);
            } else {
                int len = 0, rep;
                if (sym == 16) {
                    if (idx == 0) fail("repeat without a length");
                    len = lengths[idx - 1];
                    rep = 3 + bits(2);
                } else if (sym == 17) {
                    rep = 3 + bits(3);
                } else {
                    rep = 11 + bits(7);
                }
                if (idx + rep > nlen + ndist) fail("too many lengths");
                while (rep--) lengths[idx++] = static_cast<uint8_t>(len);
            }
        }
        if (lengths[256] == 0) fail("no end-of-block code");
        build(lc, lengths, nlen);
        build(dc, lengths + nlen, ndist);
        codes(lc, dc);
    }
};

// zlib stream (RFC 1950): header, deflate data, Adler-32 trailer.
std::vector<uint8_t> zlib_decompress(const uint8_t* in, size_t n, size_t expect) {
    if (n < 6) throw std::runtime_error("HDF5: deflate chunk too short");
    if ((in[0] & 0x0f) != 8 || ((in[0] << 8) | in[1]) % 31 != 0 || (in[1] & 0x20))
        throw std::runtime_error("HDF5: invalid zlib header in a deflate chunk");
    std::vector<uint8_t> out;
    out.reserve(expect);
    Inflate(in + 2, n - 2, out).run();
    uint32_t a = 1, b = 0;
    for (uint8_t c : out) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    const size_t end = n - 4;
    const uint32_t want = (uint32_t(in[end]) << 24) | (uint32_t(in[end + 1]) << 16) | (uint32_t(in[end + 2]) << 8) |
                          uint32_t(in[end + 3]);
    if (((b << 16) | a) != want) throw std::runtime_error("HDF5: Adler-32 mismatch in a deflate chunk");
    return out;
}

constexpr uint64_t kUndef = ~uint64_t{0};

} // namespace

namespace h5 {

// --------------------------------------------------------------- reader
void Reader::need(uint64_t at, uint64_t n) const {
    if (at > f_.size() || n > f_.size() - at) throw std::runtime_error("HDF5: truncated or corrupt file");
}

uint64_t Reader::u(uint64_t at, int n) const {
    need(at, static_cast<uint64_t>(n));
    uint64_t v = 0;
    for (int k = n - 1; k >= 0; --k) v = (v << 8) | f_[at + k];
    return v;
}

Reader::Reader(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::runtime_error("HDF5: cannot open " + path);
    f_.assign(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    uint64_t sb = kUndef;
    for (uint64_t at = 0; at + 8 <= f_.size(); at = at ? at * 2 : 512) {
        if (std::memcmp(f_.data() + at, sig, 8) == 0) {
            sb = at;
            break;
        }
    }
    if (sb == kUndef) throw std::runtime_error("HDF5: no superblock in " + path);
    const int version = static_cast<int>(u(sb + 8, 1));
    uint64_t root = kUndef;
    if (version <= 1) {
        so_ = static_cast<int>(u(sb + 13, 1));
        sl_ = static_cast<int>(u(sb + 14, 1));
        uint64_t at = sb + 24 + (version == 1 ? 4 : 0);
        base_ = u(at, so_);
        at += 4 * static_cast<uint64_t>(so_); // base, free space, end of file, driver block
        root = u(at + so_, so_);             // root symbol table entry: object header address
    } else if (version <= 3) {
        so_ = static_cast<int>(u(sb + 9, 1));
        sl_ = static_cast<int>(u(sb + 10, 1));
        const uint64_t at = sb + 12;
        base_ = u(at, so_);
        root = u(at + 3 * static_cast<uint64_t>(so_), so_); // base, extension, end of file, root header
    } else {
        throw std::runtime_error("HDF5: unsupported superblock version " + std::to_string(version));
    }
    if (so_ < 2 || so_ > 8 || sl_ < 2 || sl_ > 8) throw std::runtime_error("HDF5: unsupported offset sizes");
    read_group(base_ + root);
}

std::vector<std::string> Reader::names() const {
    std::vector<std::string> v;
    for (const auto& kv : objects_) v.push_back(kv.first);
    return v;
}

std::vector<std::array<uint64_t, 3>> Reader::messages(uint64_t at) const {
    std::vector<std::array<uint64_t, 3>> out;
    need(at, 16);
    if (std::memcmp(f_.data() + at, "OHDR", 4) == 0) {
        const int flags = static_cast<int>(u(at + 5, 1));
        uint64_t p = at + 6 + ((flags & 0x20) ? 16 : 0) + ((flags & 0x10) ? 4 : 0);
        const int sz = 1 << (flags & 3);
        const uint64_t len = u(p, sz);
        p += sz;
        std::vector<std::pair<uint64_t, uint64_t>> blocks{{p, len}};
        const int hdr = (flags & 0x04) ? 6 : 4;
        for (size_t b = 0; b < blocks.size(); ++b) {
            uint64_t q = blocks[b].first;
            const uint64_t end = q + blocks[b].second;
            while (q + hdr <= end) {
                const uint64_t type = u(q, 1), size = u(q + 1, 2);
                const uint64_t data = q + hdr;
                need(data, size);
                if (type == 0x10) { // continuation: "OCHK" block, messages, checksum
                    const uint64_t c = base_ + u(data, so_), cl = u(data + so_, sl_);
                    need(c, cl);
                    if (cl < 8 || std::memcmp(f_.data() + c, "OCHK", 4) != 0)
                        throw std::runtime_error("HDF5: bad object header continuation");
                    blocks.push_back({c + 4, cl - 8});
                } else if (type != 0) {
                    out.push_back({type, data, size});
                }
                q = data + size;
            }
        }
        return out;
    }
    if (u(at, 1) != 1) throw std::runtime_error("HDF5: unsupported object header version");
    const uint64_t nmsg = u(at + 2, 2);
    std::vector<std::pair<uint64_t, uint64_t>> blocks{{at + 16, u(at + 8, 4)}};
    uint64_t seen = 0;
    for (size_t b = 0; b < blocks.size() && seen < nmsg; ++b) {
        uint64_t q = blocks[b].first;
        const uint64_t end = q + blocks[b].second;
        while (q + 8 <= end && seen < nmsg) {
            const uint64_t type = u(q, 2), size = u(q + 2, 2);
            const uint64_t data = q + 8;
            need(data, size);
            ++seen;
            if (type == 0x10) blocks.push_back({base_ + u(data, so_), u(data + so_, sl_)});
            else if (type != 0) out.push_back({type, data, size});
            q = data + ((size + 7) & ~uint64_t{7});
        }
    }
    return out;
}

std::string Reader::heap_name(uint64_t heap_data, uint64_t offset) const {
    std::string s;
    for (uint64_t p = heap_data + offset;; ++p) {
        need(p, 1);
        if (!f_[p]) break;
        s.push_back(static_cast<char>(f_[p]));
    }
    return s;
}

void Reader::group_btree(uint64_t node, uint64_t heap_data) {
    need(node, 8);
    if (std::memcmp(f_.data() + node, "TREE", 4) != 0 || u(node + 4, 1) != 0)
        throw std::runtime_error("HDF5: bad group B-tree node");
    const int level = static_cast<int>(u(node + 5, 1));
    const int entries = static_cast<int>(u(node + 6, 2));
    uint64_t p = node + 8 + 2 * static_cast<uint64_t>(so_) + sl_; // siblings, key 0
    for (int e = 0; e < entries; ++e) {
        const uint64_t child = base_ + u(p, so_);
        p += so_ + sl_;
        if (level > 0) {
            group_btree(child, heap_data);
            continue;
        }
        need(child, 8);
        if (std::memcmp(f_.data() + child, "SNOD", 4) != 0) throw std::runtime_error("HDF5: bad symbol table node");
        const int n = static_cast<int>(u(child + 6, 2));
        uint64_t q = child + 8;
        for (int k = 0; k < n; ++k) {
            const uint64_t name = u(q, so_), header = u(q + so_, so_);
            objects_[heap_name(heap_data, name)] = base_ + header;
            q += 2 * static_cast<uint64_t>(so_) + 24;
        }
    }
}

void Reader::read_group(uint64_t header) {
    for (const auto& m : messages(header)) {
        if (m[0] == 0x11) { // symbol table: v1 B-tree and local heap
            const uint64_t btree = base_ + u(m[1], so_), heap = base_ + u(m[1] + so_, so_);
            need(heap, 8);
            if (std::memcmp(f_.data() + heap, "HEAP", 4) != 0) throw std::runtime_error("HDF5: bad local heap");
            const uint64_t data = base_ + u(heap + 8 + 2 * static_cast<uint64_t>(sl_), so_);
            group_btree(btree, data);
        } else if (m[0] == 0x06) { // link message (compact new-style group)
            uint64_t p = m[1];
            const int flags = static_cast<int>(u(p + 1, 1));
            p += 2;
            int type = 0;
            if (flags & 0x08) type = static_cast<int>(u(p++, 1));
            if (flags & 0x04) p += 8;
            if (flags & 0x10) p += 1;
            const int lsz = 1 << (flags & 3);
            const uint64_t nlen = u(p, lsz);
            p += lsz;
            need(p, nlen);
            const std::string name(reinterpret_cast<const char*>(f_.data() + p), nlen);
            p += nlen;
            if (type == 0) objects_[name] = base_ + u(p, so_);
        } else if (m[0] == 0x02) {
            throw std::runtime_error("HDF5: groups with dense link storage are not supported");
        }
    }
}

void Reader::chunk_btree(uint64_t node, int rank, std::vector<std::array<uint64_t, 3>>& chunks,
                         std::vector<std::vector<uint64_t>>& offsets) const {
    need(node, 8);
    if (std::memcmp(f_.data() + node, "TREE", 4) != 0 || u(node + 4, 1) != 1)
        throw std::runtime_error("HDF5: bad chunk B-tree node");
    const int level = static_cast<int>(u(node + 5, 1));
    const int entries = static_cast<int>(u(node + 6, 2));
    const uint64_t key = 8 + 8 * static_cast<uint64_t>(rank + 1);
    uint64_t p = node + 8 + 2 * static_cast<uint64_t>(so_);
    for (int e = 0; e < entries; ++e) {
        const uint64_t size = u(p, 4), mask = u(p + 4, 4);
        std::vector<uint64_t> off(rank);
        for (int d = 0; d < rank; ++d) off[d] = u(p + 8 + 8 * static_cast<uint64_t>(d), 8);
        const uint64_t child = base_ + u(p + key, so_);
        p += key + so_;
        if (level > 0) {
            chunk_btree(child, rank, chunks, offsets);
        } else {
            chunks.push_back({child, size, mask});
            offsets.push_back(off);
        }
    }
}

Dataset Reader::read(const std::string& name) const {
    auto it = objects_.find(name);
    if (it == objects_.end()) throw std::runtime_error("Missing HDF5 dataset: " + name);
    Dataset out;
    int dclass = -1, esize = 0;
    bool big = false, is_signed = true;
    int layout = -1;
    uint64_t addr = kUndef, csize = 0, compact_at = 0;
    std::vector<uint64_t> chunk_dims;
    struct Filter {
        int id;
        std::vector<uint32_t> client;
    };
    std::vector<Filter> filters;
    for (const auto& m : messages(it->second)) {
        const uint64_t d = m[1];
        if (m[0] == 0x01) { // dataspace
            const int v = static_cast<int>(u(d, 1)), rank = static_cast<int>(u(d + 1, 1));
            uint64_t p = d + (v == 1 ? 8 : 4);
            out.dims.resize(rank);
            for (int k = 0; k < rank; ++k) out.dims[k] = u(p + static_cast<uint64_t>(k) * sl_, sl_);
        } else if (m[0] == 0x03) { // datatype
            const uint64_t b = u(d, 1);
            dclass = static_cast<int>(b & 0x0f);
            const uint64_t bits = u(d + 1, 1);
            big = (bits & 1) != 0;
            is_signed = (bits & 0x08) != 0;
            esize = static_cast<int>(u(d + 4, 4));
        } else if (m[0] == 0x08) { // data layout
            const int v = static_cast<int>(u(d, 1));
            if (v == 3) {
                layout = static_cast<int>(u(d + 1, 1));
                if (layout == 0) {
                    csize = u(d + 2, 2);
                    compact_at = d + 4;
                } else if (layout == 1) {
                    addr = u(d + 2, so_);
                    csize = u(d + 2 + so_, sl_);
                } else if (layout == 2) {
                    const int nd = static_cast<int>(u(d + 2, 1));
                    addr = u(d + 3, so_);
                    for (int k = 0; k < nd; ++k) chunk_dims.push_back(u(d + 3 + so_ + 4 * static_cast<uint64_t>(k), 4));
                }
            } else if (v == 1 || v == 2) {
                const int nd = static_cast<int>(u(d + 1, 1));
                layout = static_cast<int>(u(d + 2, 1));
                uint64_t p = d + 8;
                if (layout != 0) {
                    addr = u(p, so_);
                    p += so_;
                }
                for (int k = 0; k < nd; ++k) chunk_dims.push_back(u(p + 4 * static_cast<uint64_t>(k), 4));
                p += 4 * static_cast<uint64_t>(nd);
                if (layout == 0) {
                    csize = u(p, 4);
                    compact_at = p + 4;
                } else if (layout == 1) {
                    csize = 0;
                    for (uint64_t c : chunk_dims) csize = csize ? csize * c : c;
                    chunk_dims.clear();
                }
            } else {
                throw std::runtime_error("HDF5: data layout version " + std::to_string(v) + " of " + name +
                                         " is not supported");
            }
        } else if (m[0] == 0x0B) { // filter pipeline
            const int v = static_cast<int>(u(d, 1)), nf = static_cast<int>(u(d + 1, 1));
            uint64_t p = d + (v == 1 ? 8 : 2);
            for (int k = 0; k < nf; ++k) {
                Filter f;
                f.id = static_cast<int>(u(p, 2));
                uint64_t namelen = 0;
                if (v == 1 || f.id >= 256) {
                    namelen = u(p + 2, 2);
                    p += 4;
                } else {
                    p += 2;
                }
                const int nc = static_cast<int>(u(p + 2, 2));
                p += 4;
                p += v == 1 ? ((namelen + 7) & ~uint64_t{7}) : namelen;
                for (int c = 0; c < nc; ++c) f.client.push_back(static_cast<uint32_t>(u(p + 4 * static_cast<uint64_t>(c), 4)));
                p += 4 * static_cast<uint64_t>(nc);
                if (v == 1 && (nc & 1)) p += 4;
                filters.push_back(f);
            }
        }
    }
    if (dclass != 0 && dclass != 1) throw std::runtime_error("Dataset " + name + " is not numeric");
    if (big) throw std::runtime_error("Dataset " + name + " is big-endian");
    if (!(esize == 1 || esize == 2 || esize == 4 || esize == 8) || (dclass == 1 && esize < 4))
        throw std::runtime_error("Dataset " + name + " has an unsupported element size");
    size_t n = 1; // a scalar (rank 0) holds one value
    for (uint64_t d : out.dims) {
        if (d == 0 || d > std::numeric_limits<size_t>::max() / n) throw std::runtime_error("Dataset " + name + " is empty or too large");
        n *= static_cast<size_t>(d);
    }
    std::vector<uint8_t> raw(n * static_cast<size_t>(esize));
    if (layout == 0 || layout == 1) {
        const uint64_t at = layout == 0 ? compact_at : base_ + addr;
        if (layout == 1 && addr == kUndef) throw std::runtime_error("Dataset " + name + " has no storage");
        need(at, raw.size());
        std::memcpy(raw.data(), f_.data() + at, raw.size());
    } else if (layout == 2) {
        const int rank = static_cast<int>(out.dims.size());
        if (rank == 0) throw std::runtime_error("Dataset " + name + " is a chunked scalar");
        if (static_cast<int>(chunk_dims.size()) != rank + 1) throw std::runtime_error("Dataset " + name + " chunk rank mismatch");
        std::vector<std::array<uint64_t, 3>> chunks;
        std::vector<std::vector<uint64_t>> offs;
        if (addr != kUndef) chunk_btree(base_ + addr, rank, chunks, offs);
        size_t per = static_cast<size_t>(esize);
        for (int d = 0; d < rank; ++d) per *= static_cast<size_t>(chunk_dims[d]);
        for (size_t c = 0; c < chunks.size(); ++c) {
            need(chunks[c][0], chunks[c][1]);
            std::vector<uint8_t> buf(f_.begin() + static_cast<std::ptrdiff_t>(chunks[c][0]),
                                     f_.begin() + static_cast<std::ptrdiff_t>(chunks[c][0] + chunks[c][1]));
            for (int k = static_cast<int>(filters.size()) - 1; k >= 0; --k) {
                if (chunks[c][2] & (1u << k)) continue; // filter skipped for this chunk
                const Filter& fl = filters[k];
                if (fl.id == 1) {
                    buf = zlib_decompress(buf.data(), buf.size(), per);
                } else if (fl.id == 2) {
                    const size_t es = fl.client.empty() ? static_cast<size_t>(esize) : fl.client[0];
                    std::vector<uint8_t> t(buf.size());
                    const size_t ne = buf.size() / es;
                    for (size_t e = 0; e < ne; ++e)
                        for (size_t b = 0; b < es; ++b) t[e * es + b] = buf[b * ne + e];
                    std::copy(buf.begin() + static_cast<std::ptrdiff_t>(ne * es), buf.end(),
                              t.begin() + static_cast<std::ptrdiff_t>(ne * es));
                    buf.swap(t);
                } else if (fl.id == 3) {
                    if (buf.size() < 4) throw std::runtime_error("HDF5: Fletcher-32 chunk too short");
                    buf.resize(buf.size() - 4);
                } else {
                    throw std::runtime_error("Dataset " + name + " uses unsupported HDF5 filter " + std::to_string(fl.id));
                }
            }
            if (buf.size() < per) throw std::runtime_error("Dataset " + name + " has a short chunk");
            // copy the chunk's in-range elements, row by row of the last axis
            std::vector<uint64_t> idx(rank, 0);
            const uint64_t last = chunk_dims[rank - 1];
            for (;;) {
                uint64_t src = 0, dst = 0;
                bool inside = true;
                for (int d = 0; d < rank; ++d) {
                    const uint64_t g = offs[c][d] + idx[d];
                    if (g >= out.dims[d] && d < rank - 1) inside = false;
                    src = src * chunk_dims[d] + idx[d];
                    dst = dst * out.dims[d] + g;
                }
                if (inside && offs[c][rank - 1] < out.dims[rank - 1]) {
                    const uint64_t cnt = std::min<uint64_t>(last, out.dims[rank - 1] - offs[c][rank - 1]);
                    std::memcpy(raw.data() + dst * esize, buf.data() + src * esize, cnt * esize);
                }
                int d = rank - 2;
                for (; d >= 0; --d) {
                    if (++idx[d] < chunk_dims[d]) break;
                    idx[d] = 0;
                }
                if (d < 0) break;
            }
        }
    } else {
        throw std::runtime_error("Dataset " + name + " has no data layout");
    }
    out.values.resize(n);
    for (size_t k = 0; k < n; ++k) {
        const uint8_t* p = raw.data() + k * static_cast<size_t>(esize);
        if (dclass == 1) {
            if (esize == 8) {
                double v;
                std::memcpy(&v, p, 8);
                out.values[k] = v;
            } else {
                float v;
                std::memcpy(&v, p, 4);
                out.values[k] = v;
            }
        } else {
            uint64_t v = 0;
            for (int b = esize - 1; b >= 0; --b) v = (v << 8) | p[b];
            if (is_signed && esize < 8 && (v >> (8 * esize - 1)) & 1u) v |= ~uint64_t{0} << (8 * esize);
            out.values[k] = is_signed ? static_cast<double>(static_cast<int64_t>(v)) : static_cast<double>(v);
        }
    }
    return out;
}

// --------------------------------------------------------------- writer
namespace {
struct Out {
    std::vector<uint8_t> b;
    void put(uint64_t v, int n) {
        for (int k = 0; k < n; ++k) b.push_back(static_cast<uint8_t>(v >> (8 * k)));
    }
    void at(size_t pos, uint64_t v, int n) {
        for (int k = 0; k < n; ++k) b[pos + k] = static_cast<uint8_t>(v >> (8 * k));
    }
    void pad8() {
        while (b.size() % 8) b.push_back(0);
    }
    void bytes(const void* p, size_t n) {
        const auto* c = static_cast<const uint8_t*>(p);
        b.insert(b.end(), c, c + n);
    }
};

// one object header message (type, data), data padded to 8 bytes
void message(Out& o, int type, const std::vector<uint8_t>& data) {
    const size_t size = (data.size() + 7) & ~size_t{7};
    o.put(static_cast<uint64_t>(type), 2);
    o.put(size, 2);
    o.put(0, 4); // flags, reserved
    o.bytes(data.data(), data.size());
    for (size_t k = data.size(); k < size; ++k) o.b.push_back(0);
}

std::vector<uint8_t> le(std::initializer_list<std::pair<uint64_t, int>> fields) {
    Out o;
    for (const auto& f : fields) o.put(f.first, f.second);
    return o.b;
}
} // namespace

void write_file(const std::string& path, const std::map<std::string, WriteSet>& sets) {
    if (sets.empty()) throw std::invalid_argument("HDF5 writer: no datasets");
    constexpr int kLeafK = 32; // symbols per symbol table node: 2K
    if (sets.size() > 2 * kLeafK) throw std::invalid_argument("HDF5 writer: too many datasets for one node");
    Out o;
    // superblock version 0 (96 bytes), end-of-file address patched at the end
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    o.bytes(sig, 8);
    o.bytes(std::vector<uint8_t>{0, 0, 0, 0, 0, 8, 8, 0}.data(), 8);
    o.put(kLeafK, 2);
    o.put(16, 2);
    o.put(0, 4);
    o.put(0, 8);      // base address
    o.put(kUndef, 8); // free space
    const size_t eof_at = o.b.size();
    o.put(0, 8);      // end of file
    o.put(kUndef, 8); // driver block
    // root symbol table entry: name offset, object header, cache type 1 (B-tree, heap)
    o.put(0, 8);
    const size_t root_hdr_at = o.b.size();
    o.put(0, 8);
    o.put(1, 4);
    o.put(0, 4);
    const size_t root_scratch = o.b.size();
    o.put(0, 8);
    o.put(0, 8);
    // local heap data: "" at 0, then the names (sorted: std::map order), 8-byte padded
    std::vector<uint8_t> heap(8, 0);
    std::vector<uint64_t> name_off;
    for (const auto& kv : sets) {
        name_off.push_back(heap.size());
        heap.insert(heap.end(), kv.first.begin(), kv.first.end());
        heap.push_back(0);
        while (heap.size() % 8) heap.push_back(0);
    }
    o.pad8();
    const uint64_t heap_hdr = o.b.size();
    o.bytes("HEAP", 4);
    o.put(0, 4); // version 0, reserved
    o.put(heap.size(), 8);
    o.put(kUndef, 8); // no free block
    const uint64_t heap_data = heap_hdr + 32;
    o.put(heap_data, 8);
    o.bytes(heap.data(), heap.size());
    // dataset object headers and data
    std::vector<uint64_t> headers;
    for (const auto& kv : sets) {
        const WriteSet& w = kv.second;
        size_t n = 1;
        for (uint64_t d : w.dims) n *= static_cast<size_t>(d);
        if (n != w.values.size() || w.dims.empty()) throw std::invalid_argument("HDF5 writer: shape of " + kv.first);
        Out msgs;
        std::vector<uint8_t> space = le({{1, 1}, {w.dims.size(), 1}, {0, 1}, {0, 1}, {0, 4}});
        for (uint64_t d : w.dims) {
            Out t;
            t.put(d, 8);
            space.insert(space.end(), t.b.begin(), t.b.end());
        }
        message(msgs, 0x01, space);
        if (w.integer) // fixed point, version 1, little-endian, signed, 8 bytes, offset 0, precision 64
            message(msgs, 0x03, le({{0x10, 1}, {0x08, 1}, {0, 1}, {0, 1}, {8, 4}, {0, 2}, {64, 2}}));
        else // IEEE double: version 1, class 1, sign bit 63, exponent 52..62 (bias 1023), mantissa 0..51
            message(msgs, 0x03, le({{0x11, 1}, {0x20, 1}, {63, 1}, {0, 1}, {8, 4}, {0, 2}, {64, 2}, {52, 1},
                                    {11, 1}, {0, 1}, {52, 1}, {1023, 4}}));
        message(msgs, 0x05, le({{2, 1}, {2, 1}, {2, 1}, {0, 1}})); // fill value v2: late alloc, never, undefined
        const size_t bytes = 8 * n;
        const size_t layout_at = msgs.b.size() + 8 + 2;
        message(msgs, 0x08, le({{3, 1}, {1, 1}, {0, 8}, {bytes, 8}}));
        o.pad8();
        const uint64_t h = o.b.size();
        headers.push_back(h);
        o.put(1, 1);
        o.put(0, 1);
        o.put(4, 2); // messages
        o.put(1, 4); // reference count
        o.put(msgs.b.size(), 4);
        o.put(0, 4); // pad to 16
        const size_t msg_base = o.b.size();
        o.bytes(msgs.b.data(), msgs.b.size());
        o.pad8();
        const uint64_t data_at = o.b.size();
        o.at(msg_base + layout_at, data_at, 8);
        for (size_t k = 0; k < n; ++k) {
            if (w.integer) o.put(static_cast<uint64_t>(static_cast<int64_t>(std::llround(w.values[k]))), 8);
            else {
                uint64_t u;
                std::memcpy(&u, &w.values[k], 8);
                o.put(u, 8);
            }
        }
    }
    // symbol table node with every dataset (sorted names)
    o.pad8();
    const uint64_t snod = o.b.size();
    o.bytes("SNOD", 4);
    o.put(1, 1);
    o.put(0, 1);
    o.put(sets.size(), 2);
    for (size_t k = 0; k < sets.size(); ++k) {
        o.put(name_off[k], 8);
        o.put(headers[k], 8);
        o.put(0, 4);
        o.put(0, 4);
        o.put(0, 8);
        o.put(0, 8);
    }
    for (size_t k = sets.size(); k < 2 * static_cast<size_t>(kLeafK); ++k) o.put(0, 40); // unused entries
    // group B-tree: one leaf entry; keys are heap offsets of "" and of the last name
    o.pad8();
    const uint64_t btree = o.b.size();
    o.bytes("TREE", 4);
    o.put(0, 1);
    o.put(0, 1);
    o.put(1, 2);
    o.put(kUndef, 8);
    o.put(kUndef, 8);
    o.put(0, 8);
    o.put(snod, 8);
    o.put(name_off.back(), 8);
    // room for the node's full 2K children and 2K + 1 keys (internal node K = 16)
    for (int k = 1; k < 2 * 16; ++k) o.put(0, 16);
    // root group object header: one symbol table message
    o.pad8();
    const uint64_t root = o.b.size();
    Out rm;
    message(rm, 0x11, le({{btree, 8}, {heap_hdr, 8}}));
    o.put(1, 1);
    o.put(0, 1);
    o.put(1, 2);
    o.put(1, 4);
    o.put(rm.b.size(), 4);
    o.put(0, 4);
    o.bytes(rm.b.data(), rm.b.size());
    o.at(root_hdr_at, root, 8);
    o.at(root_scratch, btree, 8);
    o.at(root_scratch + 8, heap_hdr, 8);
    o.at(eof_at, o.b.size(), 8);
    std::ofstream f(path, std::ios::binary | std::ios::trunc);
    if (!f) throw std::runtime_error("HDF5 writer: cannot create " + path);
    f.write(reinterpret_cast<const char*>(o.b.data()), static_cast<std::streamsize>(o.b.size()));
    if (!f) throw std::runtime_error("HDF5 writer: write failed for " + path);
}

} // namespace h5

// --------------------------------------------------------- material folders
namespace {
std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && std::isspace(static_cast<unsigned char>(s[b]))) ++b;
    while (e > b && std::isspace(static_cast<unsigned char>(s[e - 1]))) --e;
    return s.substr(b, e - b);
}
} // namespace

// src/material/MaterialDataReader.cpp:81-148: nonblank lines, scale on line 2,
// three lattice rows scaled, volume |det|, reciprocal = 2 pi inv(lattice).
void read_poscar(const std::string& path, MaterialFolder& m) {
    namespace fs = std::filesystem;
    if (!fs::exists(path)) throw std::runtime_error("POSCAR not found: " + path);
    std::ifstream in(path);
    if (!in) throw std::runtime_error("Failed to open POSCAR: " + path);
    std::vector<std::string> lines;
    for (std::string line; std::getline(in, line);) {
        const std::string t = trim(line);
        if (!t.empty()) lines.push_back(t);
    }
    if (lines.size() < 5) throw std::runtime_error("POSCAR has insufficient lines.");
    const double scale = std::stod(lines[1]);
    if (!std::isfinite(scale)) throw std::runtime_error("Non-finite POSCAR scale.");
    auto& a = m.lattice;
    for (int i = 0; i < 3; ++i) {
        std::istringstream row(lines[2 + i]);
        if (!(row >> a[i][0] >> a[i][1] >> a[i][2])) throw std::runtime_error("Failed to parse POSCAR lattice vector.");
        for (int j = 0; j < 3; ++j) {
            a[i][j] *= scale;
            if (!std::isfinite(a[i][j])) throw std::runtime_error("Non-finite POSCAR lattice.");
        }
    }
    const double det = a[0][0] * (a[1][1] * a[2][2] - a[1][2] * a[2][1]) -
                       a[0][1] * (a[1][0] * a[2][2] - a[1][2] * a[2][0]) +
                       a[0][2] * (a[1][0] * a[2][1] - a[1][1] * a[2][0]);
    m.volume_a3 = std::abs(det);
    if (!std::isfinite(m.volume_a3) || !(m.volume_a3 > 0.0)) throw std::runtime_error("POSCAR unit-cell volume is non-positive.");
    if (std::abs(det) <= 1e-20) throw std::runtime_error("Failed to invert POSCAR lattice.");
    const double id = 1.0 / det;
    const double inv[3][3] = {
        {(a[1][1] * a[2][2] - a[1][2] * a[2][1]) * id, (a[0][2] * a[2][1] - a[0][1] * a[2][2]) * id,
         (a[0][1] * a[1][2] - a[0][2] * a[1][1]) * id},
        {(a[1][2] * a[2][0] - a[1][0] * a[2][2]) * id, (a[0][0] * a[2][2] - a[0][2] * a[2][0]) * id,
         (a[0][2] * a[1][0] - a[0][0] * a[1][2]) * id},
        {(a[1][0] * a[2][1] - a[1][1] * a[2][0]) * id, (a[0][1] * a[2][0] - a[0][0] * a[2][1]) * id,
         (a[0][0] * a[1][1] - a[0][1] * a[1][0]) * id}};
    constexpr double kTwoPi = 2.0 * 3.14159265358979323846;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            m.reciprocal[i][j] = inv[i][j] * kTwoPi;
            if (!std::isfinite(m.reciprocal[i][j])) throw std::runtime_error("Non-finite reciprocal lattice.");
        }
}

MaterialFolder read_material_folder(const std::string& folder) {
    namespace fs = std::filesystem;
    MaterialFolder m;
    try {
        read_poscar((fs::path(folder) / "POSCAR").string(), m);
    } catch (const std::exception& e) {
        throw std::runtime_error(std::string("Strict POSCAR loading failed: ") + e.what());
    }
    fs::path file = fs::path(folder) / "kappa-fbz.hdf5";
    if (!fs::exists(file)) file = fs::path(folder) / "kappa.hdf5";
    if (!fs::exists(file)) {
        std::vector<fs::path> found;
        for (const auto& e : fs::directory_iterator(folder))
            if (e.is_regular_file() && e.path().extension() == ".hdf5") found.push_back(e.path());
        if (found.size() > 1) throw std::runtime_error("Ambiguous HDF5 files: provide kappa-fbz.hdf5 or kappa.hdf5.");
        if (found.size() == 1) file = found.front();
    }
    if (!fs::exists(file)) throw std::runtime_error("No HDF5 file found under material folder: " + folder);
    m.hdf5_path = file.string();
    const h5::Reader r(m.hdf5_path);
    const h5::Dataset om = r.read("frequency");
    if (om.dims.size() != 2) throw std::runtime_error("frequency rank mismatch");
    if (om.dims[0] > static_cast<uint64_t>(std::numeric_limits<int>::max()) / om.dims[1])
        throw std::runtime_error("frequency has too many modes for integer mode indices");
    m.qpoints = static_cast<int>(om.dims[0]);
    m.branches = static_cast<int>(om.dims[1]);
    m.frequency_thz = om.values;
    const h5::Dataset qp = r.read("qpoint");
    if (qp.dims.size() != 2 || qp.dims[0] != om.dims[0] || qp.dims[1] != 3) throw std::runtime_error("qpoint shape mismatch");
    m.qpoint_fractions.resize(m.qpoints);
    for (int q = 0; q < m.qpoints; ++q)
        for (int k = 0; k < 3; ++k) m.qpoint_fractions[q][k] = qp.values[3 * static_cast<size_t>(q) + k];
    const h5::Dataset mesh = r.read("mesh");
    if (mesh.dims.size() != 1 || mesh.dims[0] != 3) throw std::runtime_error("mesh must have shape (3)");
    for (int a = 0; a < 3; ++a) {
        const double c = mesh.values[a];
        if (!std::isfinite(c) || c < 1 || c != std::floor(c) || c > std::numeric_limits<int>::max())
            throw std::runtime_error("mesh entries must be positive integers");
        m.mesh[a] = static_cast<int>(c);
    }
    if (r.has("weight")) {
        const h5::Dataset w = r.read("weight");
        if (w.dims.size() != 1 || w.dims[0] != om.dims[0] ||
            std::any_of(w.values.begin(), w.values.end(), [](double x) { return x != 1.0; }))
            throw std::runtime_error("Full Brillouin-zone data requires one unit weight per qpoint");
    }
    const h5::Dataset gv = r.read("group_velocity");
    if (gv.dims.size() != 3 || gv.dims[0] != om.dims[0] || gv.dims[1] != om.dims[1] || gv.dims[2] != 3)
        throw std::runtime_error("group_velocity shape mismatch");
    const size_t nm = static_cast<size_t>(m.qpoints) * m.branches;
    m.group_velocity.resize(nm);
    for (size_t i = 0; i < nm; ++i)
        for (int k = 0; k < 3; ++k) m.group_velocity[i][k] = gv.values[3 * i + k];
    const h5::Dataset T = r.read("temperature");
    if (T.dims.size() != 1) throw std::runtime_error("temperature rank mismatch");
    m.temperatures = T.values;
    const h5::Dataset g = r.read("gamma");
    if (g.dims.size() != 3 || g.dims[0] != T.values.size() || g.dims[1] != om.dims[0] || g.dims[2] != om.dims[1])
        throw std::runtime_error("gamma shape mismatch");
    m.gamma = g.values;
    for (const auto& e : {std::make_pair("gamma_N", &m.gamma_normal), std::make_pair("gamma_U", &m.gamma_umklapp)}) {
        if (!r.has(e.first)) continue;
        const h5::Dataset d = r.read(e.first);
        if (d.dims != g.dims) throw std::runtime_error(std::string(e.first) + " shape mismatch");
        *e.second = d.values;
    }
    for (const char* name : {"gamma_isotope", "gamma_impurity", "gamma_defect"}) {
        if (!r.has(name)) continue;
        const h5::Dataset d = r.read(name);
        if (d.dims != om.dims && d.dims != g.dims)
            throw std::runtime_error(std::string(name) + " shape mismatch: expected (q, branch) or (temperature, q, branch)");
        m.gamma_resistive[name] = d.values;
    }
    return m;
}

void write_material_folder(const std::string& folder, const MaterialFolder& m) {
    namespace fs = std::filesystem;
    fs::create_directories(folder);
    auto a = m.lattice;
    bool have = false;
    for (const auto& row : a)
        for (double x : row) have = have || x != 0.0;
    if (!have) { // lattice = 2 pi inv(reciprocal)
        const auto& b = m.reciprocal;
        const double det = b[0][0] * (b[1][1] * b[2][2] - b[1][2] * b[2][1]) -
                           b[0][1] * (b[1][0] * b[2][2] - b[1][2] * b[2][0]) +
                           b[0][2] * (b[1][0] * b[2][1] - b[1][1] * b[2][0]);
        if (!(std::abs(det) > 0.0)) throw std::invalid_argument("material folder: singular reciprocal lattice");
        const double s = 2.0 * 3.14159265358979323846 / det;
        a = {{{(b[1][1] * b[2][2] - b[1][2] * b[2][1]) * s, (b[0][2] * b[2][1] - b[0][1] * b[2][2]) * s,
               (b[0][1] * b[1][2] - b[0][2] * b[1][1]) * s},
              {(b[1][2] * b[2][0] - b[1][0] * b[2][2]) * s, (b[0][0] * b[2][2] - b[0][2] * b[2][0]) * s,
               (b[0][2] * b[1][0] - b[0][0] * b[1][2]) * s},
              {(b[1][0] * b[2][1] - b[1][1] * b[2][0]) * s, (b[0][1] * b[2][0] - b[0][0] * b[2][1]) * s,
               (b[0][0] * b[1][1] - b[0][1] * b[1][0]) * s}}};
    }
    {
        std::ofstream p((fs::path(folder) / "POSCAR").string(), std::ios::trunc);
        if (!p) throw std::runtime_error("material folder: cannot write POSCAR in " + folder);
        p << "synthetic phonon table\n1.0\n" << std::setprecision(17);
        for (const auto& row : a) p << row[0] << ' ' << row[1] << ' ' << row[2] << '\n';
        p << "X\n1\nDirect\n0.0 0.0 0.0\n";
    }
    const uint64_t nq = static_cast<uint64_t>(m.qpoints), nb = static_cast<uint64_t>(m.branches);
    const uint64_t nT = m.temperatures.size();
    std::map<std::string, h5::WriteSet> sets;
    sets["frequency"] = {{nq, nb}, m.frequency_thz, false};
    std::vector<double> qp, gv;
    for (const auto& q : m.qpoint_fractions) qp.insert(qp.end(), q.begin(), q.end());
    for (const auto& v : m.group_velocity) gv.insert(gv.end(), v.begin(), v.end());
    sets["qpoint"] = {{nq, 3}, qp, false};
    sets["mesh"] = {{3}, {double(m.mesh[0]), double(m.mesh[1]), double(m.mesh[2])}, true};
    sets["weight"] = {{nq}, std::vector<double>(nq, 1.0), true};
    sets["group_velocity"] = {{nq, nb, 3}, gv, false};
    sets["temperature"] = {{nT}, m.temperatures, false};
    sets["gamma"] = {{nT, nq, nb}, m.gamma, false};
    if (!m.gamma_normal.empty()) sets["gamma_N"] = {{nT, nq, nb}, m.gamma_normal, false};
    if (!m.gamma_umklapp.empty()) sets["gamma_U"] = {{nT, nq, nb}, m.gamma_umklapp, false};
    for (const auto& kv : m.gamma_resistive) {
        const bool per_T = kv.second.size() == nT * nq * nb;
        sets[kv.first] = {per_T ? std::vector<uint64_t>{nT, nq, nb} : std::vector<uint64_t>{nq, nb}, kv.second, false};
    }
    h5::write_file((fs::path(folder) / "kappa-fbz.hdf5").string(), sets);
}

} // namespace phmc
