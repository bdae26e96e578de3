// PNG decoding to RGBA8 for the blue-noise asset.
//
// The reference decodes assets/blue_noise.png with lodepng into RGBA8
// (renderer.ixx:101-110: lodepng::decode(pixels, w, h, path, LCT_RGBA, 8))
// and uploads it as an R8G8B8A8 texture.  lodepng is an un-vendored
// dependency of the reference, so this module decodes the same files on its
// own: the zlib container (RFC 1950) around a DEFLATE stream (RFC 1951) --
// stored, fixed-Huffman and dynamic-Huffman blocks, decoded with canonical
// Huffman codes -- and the PNG scanline filters (PNG specification, 2nd
// ed., clause 9: None, Sub, Up, Average, Paeth), for 8-bit, non-interlaced
// greyscale, greyscale + alpha, RGB and RGBA images.  Chunk CRC-32s and the
// zlib Adler-32 are checked.  Channels are widened to RGBA8 the way
// LCT_RGBA does: grey g -> (g, g, g), missing alpha -> 255.
#include "mrt_host.h"

#include <cstdio>
#include <cstring>
#include <vector>

namespace {

// ------------------------------------------------------------ checksums

uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
    static uint32_t table[256];
    static bool ready = false;
    if (!ready) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        ready = true;
    }
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFFu] ^ (crc >> 8);
    return ~crc;
}

uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; ++i) {
        a = (a + p[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

uint32_t be32(const uint8_t* p) {
    return (uint32_t(p[0]) << 24) | (uint32_t(p[1]) << 16) | (uint32_t(p[2]) << 8) | uint32_t(p[3]);
}

// ------------------------------------------------------------- inflate

struct Bits {
    const uint8_t* p;
    size_t n;
    size_t pos = 0;   // byte
    uint32_t bit = 0; // bit within the byte, LSB first
    bool over = false;

    uint32_t get(uint32_t count) {  // count <= 16
        uint32_t v = 0;
        for (uint32_t k = 0; k < count; ++k) {
            if (pos >= n) {
                over = true;
                return 0;
            }
            v |= uint32_t((p[pos] >> bit) & 1u) << k;
            if (++bit == 8) {
                bit = 0;
                ++pos;
            }
        }
        return v;
    }
    void align() {
        if (bit) {
            bit = 0;
            ++pos;
        }
    }
};

// Canonical Huffman code over up to 288 symbols, lengths up to 15 bits:
// count[l] codes of length l; sym lists the symbols by (length, value).
struct Huffman {
    uint16_t count[16];
    uint16_t sym[320];

    // false when the lengths over-subscribe the code space
    bool build(const uint8_t* len, int nsym) {
        std::memset(count, 0, sizeof(count));
        for (int s = 0; s < nsym; ++s) ++count[len[s]];
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {
            left = 2 * left - count[l];
            if (left < 0) return false;
        }
        uint16_t first[16];
        first[1] = 0;
        for (int l = 1; l < 15; ++l) first[l + 1] = uint16_t(first[l] + count[l]);
        for (int s = 0; s < nsym; ++s)
            if (len[s]) sym[first[len[s]]++] = uint16_t(s);
        return true;
    }

    // next symbol, reading the code MSB-first one bit at a time; -1 on a
    // code that is not in the table or past the end of the data
    int decode(Bits& b) const {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= int(b.get(1));
            if (b.over) return -1;
            const int c = count[l];
            if (code - first < c) return sym[index + code - first];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

// RFC 1951, 3.2.5: base lengths / distances and their extra bits
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// order of the code-length code lengths in a dynamic block header (3.2.7)
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

bool inflate_codes(Bits& b, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out, size_t limit) {
    for (;;) {
        const int s = lit.decode(b);
        if (s < 0) return false;
        if (s < 256) {
            if (out.size() >= limit) return false;
            out.push_back(uint8_t(s));
        } else if (s == 256) {
            return true;
        } else {
            const int li = s - 257;
            if (li >= 29) return false;
            const uint32_t len = kLenBase[li] + b.get(kLenExtra[li]);
            const int di = dist.decode(b);
            if (di < 0 || di >= 30) return false;
            const uint32_t d = kDistBase[di] + b.get(kDistExtra[di]);
            if (b.over || d > out.size() || out.size() + len > limit) return false;
            const size_t from = out.size() - d;
            for (uint32_t k = 0; k < len; ++k) out.push_back(out[from + k]);  // may overlap itself
        }
    }
}

// Inflates a zlib stream; `limit` bounds the output (the image size).
bool zlib_inflate(const uint8_t* p, size_t n, std::vector<uint8_t>& out, size_t limit) {
    if (n < 6) return false;
    const uint32_t cmf = p[0], flg = p[1];
    if ((cmf & 15u) != 8u || (cmf >> 4) > 7u || ((cmf << 8) | flg) % 31u != 0u || (flg & 0x20u)) return false;
    Bits b{p + 2, n - 2};
    bool last = false;
    while (!last) {
        last = b.get(1) != 0;
        const uint32_t type = b.get(2);
        if (b.over) return false;
        if (type == 0) {  // stored
            b.align();
            if (b.pos + 4 > b.n) return false;
            const uint32_t len = b.p[b.pos] | (uint32_t(b.p[b.pos + 1]) << 8);
            const uint32_t nlen = b.p[b.pos + 2] | (uint32_t(b.p[b.pos + 3]) << 8);
            if ((len ^ 0xFFFFu) != nlen) return false;
            b.pos += 4;
            if (b.pos + len > b.n || out.size() + len > limit) return false;
            out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {  // fixed Huffman codes (3.2.6)
            uint8_t len[288];
            for (int s = 0; s < 288; ++s) len[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
            Huffman lit, dist;
            lit.build(len, 288);
            uint8_t dl[30];
            std::memset(dl, 5, sizeof(dl));
            dist.build(dl, 30);
            if (!inflate_codes(b, lit, dist, out, limit)) return false;
        } else if (type == 2) {  // dynamic Huffman codes (3.2.7)
            const uint32_t hlit = b.get(5) + 257, hdist = b.get(5) + 1, hclen = b.get(4) + 4;
            if (b.over || hlit > 286 || hdist > 30) return false;
            uint8_t cl[19] = {0};
            for (uint32_t k = 0; k < hclen; ++k) cl[kClOrder[k]] = uint8_t(b.get(3));
            Huffman clh;
            if (!clh.build(cl, 19)) return false;
            uint8_t len[320] = {0};
            uint32_t k = 0;
            while (k < hlit + hdist) {
                const int s = clh.decode(b);
                if (s < 0) return false;
                if (s < 16) {
                    len[k++] = uint8_t(s);
                    continue;
                }
                uint32_t rep = 0;
                uint8_t v = 0;
                if (s == 16) {
                    if (k == 0) return false;
                    v = len[k - 1];
                    rep = 3 + b.get(2);
                } else if (s == 17) {
                    rep = 3 + b.get(3);
                } else {
                    rep = 11 + b.get(7);
                }
                if (b.over || k + rep > hlit + hdist) return false;
                while (rep--) len[k++] = v;
            }
            if (len[256] == 0) return false;  // no end-of-block code
            Huffman lit, dist;
            if (!lit.build(len, int(hlit)) || !dist.build(len + hlit, int(hdist))) return false;
            if (!inflate_codes(b, lit, dist, out, limit)) return false;
        } else {
            return false;
        }
    }
    b.align();
    if (b.pos + 4 > b.n) return false;
    return be32(b.p + b.pos) == adler32(out.data(), out.size());
}

// ----------------------------------------------------------------- PNG

int paeth(int a, int b, int c) {
    const int p = a + b - c;
    const int pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

int decode(const uint8_t* data, size_t size, std::vector<uint8_t>* rgba, uint32_t* w_out, uint32_t* h_out) {
    static const uint8_t kSig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    if (!data || size < 8 + 25 || std::memcmp(data, kSig, 8) != 0) return MRT_EINVAL;
    uint32_t w = 0, h = 0, channels = 0;
    std::vector<uint8_t> idat;
    bool have_ihdr = false, have_iend = false;
    size_t pos = 8;
    while (pos + 12 <= size && !have_iend) {
        const uint32_t len = be32(data + pos);
        if (len > size - pos - 12) return MRT_EINVAL;
        const uint8_t* type = data + pos + 4;
        const uint8_t* body = data + pos + 8;
        if (crc32_update(0, type, size_t(len) + 4) != be32(body + len)) return MRT_EINVAL;
        if (!std::memcmp(type, "IHDR", 4)) {
            if (len != 13) return MRT_EINVAL;
            w = be32(body);
            h = be32(body + 4);
            const uint8_t depth = body[8], ctype = body[9];
            if (depth != 8 || body[10] != 0 || body[11] != 0 || body[12] != 0) return MRT_EINVAL;  // 8-bit, no interlace
            channels = ctype == 0 ? 1u : ctype == 4 ? 2u : ctype == 2 ? 3u : ctype == 6 ? 4u : 0u;
            if (!channels || w == 0 || h == 0 || w > (1u << 15) || h > (1u << 15)) return MRT_EINVAL;
            have_ihdr = true;
        } else if (!std::memcmp(type, "IDAT", 4)) {
            if (!have_ihdr) return MRT_EINVAL;
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            have_iend = true;
        } else if (!(type[0] & 0x20u)) {
            return MRT_EINVAL;  // an unknown critical chunk (PLTE: palette images are not read)
        }
        pos += size_t(len) + 12;
    }
    if (!have_ihdr || !have_iend || idat.empty()) return MRT_EINVAL;
    *w_out = w;
    *h_out = h;
    if (!rgba) return MRT_OK;
    const size_t stride = size_t(w) * channels;
    const size_t raw_size = (stride + 1) * h;
    std::vector<uint8_t> raw;
    raw.reserve(raw_size);
    if (!zlib_inflate(idat.data(), idat.size(), raw, raw_size) || raw.size() != raw_size) return MRT_EINVAL;
    // unfilter in place, row by row
    const int bpp = int(channels);
    for (uint32_t y = 0; y < h; ++y) {
        uint8_t* row = raw.data() + y * (stride + 1);
        const uint8_t filter = row[0];
        uint8_t* cur = row + 1;
        const uint8_t* up = y ? raw.data() + (y - 1) * (stride + 1) + 1 : nullptr;
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= size_t(bpp) ? cur[i - bpp] : 0;
            const int b = up ? up[i] : 0;
            const int c = (up && i >= size_t(bpp)) ? up[i - bpp] : 0;
            int pred = 0;
            switch (filter) {
            case 0: pred = 0; break;
            case 1: pred = a; break;
            case 2: pred = b; break;
            case 3: pred = (a + b) >> 1; break;
            case 4: pred = paeth(a, b, c); break;
            default: return MRT_EINVAL;
            }
            cur[i] = uint8_t(cur[i] + pred);
        }
    }
    rgba->resize(size_t(w) * h * 4);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t* src = raw.data() + y * (stride + 1) + 1;
        uint8_t* dst = rgba->data() + size_t(y) * w * 4;
        for (uint32_t x = 0; x < w; ++x, src += channels, dst += 4) {
            if (channels <= 2) {
                dst[0] = dst[1] = dst[2] = src[0];
                dst[3] = channels == 2 ? src[1] : 255;
            } else {
                dst[0] = src[0];
                dst[1] = src[1];
                dst[2] = src[2];
                dst[3] = channels == 4 ? src[3] : 255;
            }
        }
    }
    return MRT_OK;
}

int decode_into(const uint8_t* data, size_t size, uint8_t* out, size_t out_bytes, uint32_t* w, uint32_t* h) {
    if (!w || !h) return MRT_EINVAL;
    if (!out) return decode(data, size, nullptr, w, h);
    uint32_t hw = 0, hh = 0;
    int rc = decode(data, size, nullptr, &hw, &hh);
    if (rc != MRT_OK) return rc;
    if (out_bytes < size_t(hw) * hh * 4) return MRT_ERANGE;
    std::vector<uint8_t> img;
    rc = decode(data, size, &img, w, h);
    if (rc != MRT_OK) return rc;
    std::memcpy(out, img.data(), img.size());
    return MRT_OK;
}

} // namespace

extern "C" int mrt_png_decode_rgba8(const uint8_t* data, size_t size, uint8_t* rgba, size_t rgba_bytes,
                                    uint32_t* width, uint32_t* height) {
    return decode_into(data, size, rgba, rgba_bytes, width, height);
}

extern "C" int mrt_png_load_rgba8(const char* path, uint8_t* rgba, size_t rgba_bytes, uint32_t* width,
                                  uint32_t* height) {
    if (!path) return MRT_EINVAL;
    std::FILE* f = std::fopen(path, "rb");
    if (!f) return MRT_EINVAL;
    std::vector<uint8_t> data;
    uint8_t buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f)) > 0) data.insert(data.end(), buf, buf + got);
    std::fclose(f);
    return decode_into(data.data(), data.size(), rgba, rgba_bytes, width, height);
}
