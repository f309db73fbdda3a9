// instance_io.cpp -- graph-matching instance files: MATLAB v5 matrices
// (the reference's examples/main.cu:41-129 loader: a named miMATRIX, possibly
// inside a zlib-compressed miCOMPRESSED element) and DIMACS edge lists
// ("p edge n m", "e u v" with 1-based vertices), as host arrays.
//
// The zlib stream is decoded here (RFC 1950 wrapper, RFC 1951 DEFLATE:
// stored, fixed-Huffman and dynamic-Huffman blocks, canonical codes decoded
// bit by bit), so the library needs no compression library at build time.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gpuboscia_gb300.h"

namespace gbx {
void set_last_error(const std::string& msg);
}

namespace {

// ----------------------------------------------------------------- inflate
class BitReader {
public:
    BitReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}
    int bit() {
        if (pos_ >= n_) throw std::runtime_error("deflate stream truncated");
        const int b = (p_[pos_] >> nbit_) & 1;
        if (++nbit_ == 8) { nbit_ = 0; ++pos_; }
        return b;
    }
    unsigned bits(int count) {   // LSB first
        unsigned v = 0;
        for (int i = 0; i < count; ++i) v |= (unsigned)bit() << i;
        return v;
    }
    void align() { if (nbit_) { nbit_ = 0; ++pos_; } }
    size_t pos() const { return pos_; }
    void skip(size_t k) { pos_ += k; }
    const uint8_t* at() const { return p_ + pos_; }
    size_t left() const { return n_ - pos_; }

private:
    const uint8_t* p_;
    size_t n_;
    size_t pos_ = 0;
    int nbit_ = 0;
};

// canonical Huffman code: number of codes per length, symbols in code order
struct Huffman {
    std::vector<int> count = std::vector<int>(16, 0);
    std::vector<int> symbol;

    void build(const int* lengths, int n) {
        std::fill(count.begin(), count.end(), 0);
        for (int s = 0; s < n; ++s) ++count[lengths[s]];
        count[0] = 0;
        std::vector<int> offs(16, 0);
        for (int l = 1; l < 16; ++l) offs[l] = offs[l - 1] + count[l - 1];
        symbol.assign(n, 0);
        for (int s = 0; s < n; ++s)
            if (lengths[s]) symbol[offs[lengths[s]]++] = s;
    }
    int decode(BitReader& br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= br.bit();
            const int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw std::runtime_error("invalid Huffman code in deflate stream");
    }
};

// RFC 1951 section 3.2.5: length and distance base values and extra bits
const int kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115,
                          131, 163, 195, 227, 258};
const int kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const int kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537,
                           2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const int kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12,
                            13, 13};

void inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out) {
    for (;;) {
        const int s = lit.decode(br);
        if (s < 256) { out.push_back((uint8_t)s); continue; }
        if (s == 256) return;
        const int li = s - 257;
        if (li >= 29) throw std::runtime_error("invalid length symbol in deflate stream");
        const int len = kLenBase[li] + (int)br.bits(kLenExtra[li]);
        const int di = dist.decode(br);
        if (di >= 30) throw std::runtime_error("invalid distance symbol in deflate stream");
        const size_t d = (size_t)kDistBase[di] + br.bits(kDistExtra[di]);
        if (d > out.size()) throw std::runtime_error("deflate distance before the start of the output");
        const size_t from = out.size() - d;
        for (int k = 0; k < len; ++k) {
            const uint8_t b = out[from + k];   // copied before the vector may grow
            out.push_back(b);
        }
    }
}

std::vector<uint8_t> zlib_inflate(const uint8_t* p, size_t n) {
    if (n < 6) throw std::runtime_error("zlib stream too short");
    const int cmf = p[0], flg = p[1];
    if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20))
        throw std::runtime_error("unsupported zlib header");
    BitReader br(p + 2, n - 2);
    std::vector<uint8_t> out;
    bool last = false;
    while (!last) {
        last = br.bit() != 0;
        const unsigned type = br.bits(2);
        if (type == 0) {
            br.align();
            if (br.left() < 4) throw std::runtime_error("stored block truncated");
            const uint8_t* h = br.at();
            const unsigned len = h[0] | (h[1] << 8), nlen = h[2] | (h[3] << 8);
            if ((len ^ 0xffffu) != nlen) throw std::runtime_error("stored block length mismatch");
            br.skip(4);
            if (br.left() < len) throw std::runtime_error("stored block truncated");
            out.insert(out.end(), br.at(), br.at() + len);
            br.skip(len);
        } else if (type == 1) {
            // the fixed code of RFC 1951 section 3.2.6
            Huffman lit, dist;
            int l[288], d[30];
            for (int s = 0; s < 288; ++s) l[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
            for (int s = 0; s < 30; ++s) d[s] = 5;
            lit.build(l, 288);
            dist.build(d, 30);
            inflate_block(br, lit, dist, out);
        } else if (type == 2) {
            const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            static const int order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            int cl[19] = {0};
            for (int i = 0; i < hclen; ++i) cl[order[i]] = (int)br.bits(3);
            Huffman clh;
            clh.build(cl, 19);
            std::vector<int> lens(hlit + hdist, 0);
            for (int i = 0; i < hlit + hdist;) {
                const int s = clh.decode(br);
                if (s < 16) { lens[i++] = s; continue; }
                int rep = 0, val = 0;
                if (s == 16) {
                    if (i == 0) throw std::runtime_error("repeat with no previous length");
                    val = lens[i - 1];
                    rep = 3 + (int)br.bits(2);
                } else if (s == 17) {
                    rep = 3 + (int)br.bits(3);
                } else {
                    rep = 11 + (int)br.bits(7);
                }
                if (i + rep > hlit + hdist) throw std::runtime_error("code lengths overflow");
                while (rep--) lens[i++] = val;
            }
            Huffman lit, dist;
            lit.build(lens.data(), hlit);
            dist.build(lens.data() + hlit, hdist);
            inflate_block(br, lit, dist, out);
        } else {
            throw std::runtime_error("invalid deflate block type");
        }
    }
    // Adler-32 of the output (RFC 1950)
    br.align();
    if (br.left() >= 4) {
        uint32_t a = 1, b = 0;
        for (uint8_t v : out) { a = (a + v) % 65521u; b = (b + a) % 65521u; }
        const uint8_t* t = br.at();
        const uint32_t want = ((uint32_t)t[0] << 24) | ((uint32_t)t[1] << 16) | ((uint32_t)t[2] << 8) | t[3];
        if (want != ((b << 16) | a)) throw std::runtime_error("zlib checksum mismatch");
    }
    return out;
}

// ----------------------------------------------------------------- MAT v5
struct Element {
    uint32_t type = 0, bytes = 0;
    const uint8_t* data = nullptr;
};

uint32_t u32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

// one data element; small elements pack tag and data into 8 bytes
Element next(const uint8_t*& p, const uint8_t* end) {
    if (end - p < 8) throw std::runtime_error("truncated MAT element");
    const uint32_t tag = u32(p);
    Element e;
    if (tag >> 16) {
        e.type = tag & 0xffffu;
        e.bytes = tag >> 16;
        e.data = p + 4;
        p += 8;
        return e;
    }
    e.type = tag;
    e.bytes = u32(p + 4);
    e.data = p + 8;
    // compressed elements are not padded to 8 bytes by every writer
    const size_t stored = e.type == 15 ? e.bytes : (e.bytes + 7u) & ~size_t(7);
    if ((size_t)(end - e.data) < e.bytes) throw std::runtime_error("truncated MAT payload");
    p = e.data + std::min<size_t>(stored, (size_t)(end - e.data));
    return e;
}

double numeric_at(const Element& e, size_t k) {
    const uint8_t* d = e.data;
    switch (e.type) {
    case 1: return (double)(int8_t)d[k];
    case 2: return (double)d[k];
    case 3: { int16_t v; std::memcpy(&v, d + 2 * k, 2); return v; }
    case 4: { uint16_t v; std::memcpy(&v, d + 2 * k, 2); return v; }
    case 5: { int32_t v; std::memcpy(&v, d + 4 * k, 4); return v; }
    case 6: { uint32_t v; std::memcpy(&v, d + 4 * k, 4); return v; }
    case 7: { float v; std::memcpy(&v, d + 4 * k, 4); return v; }
    case 9: { double v; std::memcpy(&v, d + 8 * k, 8); return v; }
    case 12: { int64_t v; std::memcpy(&v, d + 8 * k, 8); return (double)v; }
    case 13: { uint64_t v; std::memcpy(&v, d + 8 * k, 8); return (double)v; }
    default: throw std::runtime_error("unsupported MAT numeric type " + std::to_string(e.type));
    }
}

size_t type_size(uint32_t t) {
    switch (t) {
    case 1: case 2: return 1;
    case 3: case 4: return 2;
    case 5: case 6: case 7: return 4;
    case 9: case 12: case 13: return 8;
    default: return 0;
    }
}

// A miMATRIX payload; fills out (row-major) when its name is `wanted`.
bool parse_matrix(const uint8_t* p, const uint8_t* end, const std::string& wanted, int* rows, int* cols,
                  std::vector<double>* out) {
    const Element flags = next(p, end);
    if (flags.bytes < 8) throw std::runtime_error("invalid MAT array flags");
    const int cls = (int)(u32(flags.data) & 0xff);
    const bool complex_ = (u32(flags.data) >> 11) & 1;
    const Element dims = next(p, end);
    if (dims.bytes != 8) return false;   // only two-dimensional arrays
    const Element name = next(p, end);
    if (std::string((const char*)name.data, name.bytes) != wanted) return false;
    if (cls == 5) throw std::runtime_error("sparse MAT matrices are not supported; save A as full");
    if (cls < 6 || cls > 15 || complex_) throw std::runtime_error("MAT variable is not a real numeric matrix");
    int32_t r, c;
    std::memcpy(&r, dims.data, 4);
    std::memcpy(&c, dims.data + 4, 4);
    if (r < 0 || c < 0) throw std::runtime_error("invalid MAT dimensions");
    const Element real = next(p, end);
    const size_t ts = type_size(real.type), count = (size_t)r * c;
    if (!ts || real.bytes < count * ts) throw std::runtime_error("MAT data shorter than its dimensions");
    out->assign(count, 0.0);
    for (int j = 0; j < c; ++j)        // column-major in the file
        for (int i = 0; i < r; ++i) (*out)[(size_t)i * c + j] = numeric_at(real, (size_t)j * r + i);
    *rows = r;
    *cols = c;
    return true;
}

std::vector<double> read_mat(const std::string& path, const std::string& wanted, int* rows, int* cols) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw std::invalid_argument("cannot open " + path);
    const std::vector<uint8_t> file((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    if (file.size() < 128 || file[126] != 'I' || file[127] != 'M')
        throw std::runtime_error("not a little-endian MAT v5 file: " + path);
    const uint8_t* p = file.data() + 128;
    const uint8_t* end = file.data() + file.size();
    std::vector<double> out;
    while (end - p >= 8) {
        const Element e = next(p, end);
        if (e.type == 15) {
            const std::vector<uint8_t> raw = zlib_inflate(e.data, e.bytes);
            const uint8_t* q = raw.data();
            const Element m = next(q, raw.data() + raw.size());
            if (m.type == 14 && parse_matrix(m.data, m.data + m.bytes, wanted, rows, cols, &out)) return out;
        } else if (e.type == 14) {
            if (parse_matrix(e.data, e.data + e.bytes, wanted, rows, cols, &out)) return out;
        }
    }
    throw std::invalid_argument("MAT file has no real matrix named '" + wanted + "': " + path);
}

// ----------------------------------------------------------------- DIMACS
std::vector<double> read_dimacs(const std::string& path, int* n_out) {
    std::ifstream in(path);
    if (!in) throw std::invalid_argument("cannot open " + path);
    std::string line;
    int n = -1;
    long long m = -1, seen = 0;
    std::vector<double> A;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == 'c') continue;
        std::istringstream ss(line);
        std::string tag;
        ss >> tag;
        if (tag == "p") {
            std::string kind;
            ss >> kind >> n >> m;
            if (!ss || n <= 0 || n > 65536 || m < 0) throw std::runtime_error("invalid DIMACS problem line: " + line);
            A.assign((size_t)n * n, 0.0);
        } else if (tag == "e") {
            long long u, v;
            ss >> u >> v;
            if (n < 0) throw std::runtime_error("DIMACS edge before the problem line");
            if (!ss || u < 1 || v < 1 || u > n || v > n) throw std::runtime_error("invalid DIMACS edge: " + line);
            A[(size_t)(u - 1) * n + (v - 1)] = 1.0;
            A[(size_t)(v - 1) * n + (u - 1)] = 1.0;
            ++seen;
        }
    }
    if (n < 0) throw std::runtime_error("DIMACS file has no problem line: " + path);
    if (seen != m) throw std::runtime_error("DIMACS edge count differs from the problem line: " + path);
    *n_out = n;
    return A;
}

int finish(const std::vector<double>& v, double* out, size_t capacity) {
    if (!out) return GBX_OK;
    if (capacity < v.size()) {
        gbx::set_last_error("output buffer smaller than the matrix");
        return GBX_ERR_INVALID;
    }
    std::copy(v.begin(), v.end(), out);
    return GBX_OK;
}

}  // namespace

extern "C" {

int gbx_read_mat(const char* path, const char* name, int* rows, int* cols, double* out, size_t capacity) {
    try {
        if (!path || !rows || !cols) throw std::invalid_argument("null argument");
        const std::vector<double> v = read_mat(path, name ? name : "A", rows, cols);
        return finish(v, out, capacity);
    } catch (const std::invalid_argument& e) {
        gbx::set_last_error(e.what());
        return GBX_ERR_INVALID;
    } catch (const std::exception& e) {
        gbx::set_last_error(e.what());
        return GBX_ERR_UNSUPPORTED;
    }
}

int gbx_read_dimacs(const char* path, int* n_vertices, double* out, size_t capacity) {
    try {
        if (!path || !n_vertices) throw std::invalid_argument("null argument");
        const std::vector<double> v = read_dimacs(path, n_vertices);
        return finish(v, out, capacity);
    } catch (const std::invalid_argument& e) {
        gbx::set_last_error(e.what());
        return GBX_ERR_INVALID;
    } catch (const std::exception& e) {
        gbx::set_last_error(e.what());
        return GBX_ERR_UNSUPPORTED;
    }
}

}  // extern "C"
