// assets.cpp - loader for the reference's shipped texture assets (Texture.cpp:212-246 and
// 502-538 with stb_image's stbi_load(..., STBI_rgb_alpha)): TGA (uncompressed or run-length
// encoded, 8-bit grey or 24/32-bit BGR(A), either row order) and PNG (8- or 16-bit grey,
// grey+alpha, RGB or RGBA, not interlaced), decoded to RGBA8 rows top to bottom.
//
// Conversions match stbi_load with 4 requested channels: grey g -> (g, g, g, 255); a missing alpha
// -> 255; 16-bit samples -> their high byte (stb's 16 -> 8 bit reduction); TGA rows flipped unless
// the descriptor's top-left-origin bit (0x20) is set; a PNG tRNS colour key makes matching pixels
// transparent.
//
// PNG's zlib stream is decoded by an inflate written here from RFC 1950 / RFC 1951 (stored, fixed
// and dynamic Huffman blocks; canonical Huffman codes decoded by code length), with the PNG chunk
// CRC-32 and the zlib Adler-32 checked.
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "mm_internal.h"

namespace {

using Bytes = std::vector<uint8_t>;

bool read_file(const char* path, Bytes* out) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    out->clear();
    uint8_t buf[1 << 16];
    size_t n;
    while ((n = fread(buf, 1, sizeof(buf), f)) > 0) out->insert(out->end(), buf, buf + n);
    const bool ok = !ferror(f);
    fclose(f);
    return ok;
}

// ------------------------------------------------------------------------------ inflate (RFC 1951)

struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool over = false;
    int bit() {
        if (cnt == 0) {
            if (pos >= n) {
                over = true;
                return 0;
            }
            buf = p[pos++];
            cnt = 8;
        }
        const int b = buf & 1;
        buf >>= 1;
        --cnt;
        return b;
    }
    uint32_t bits(int k) {  // k <= 16, least significant bit first
        uint32_t v = 0;
        for (int i = 0; i < k; ++i) v |= (uint32_t)bit() << i;
        return v;
    }
    void align() { cnt = 0; }
};

// Canonical Huffman code: symbols ordered by (length, value); count[len] codes of each length.
struct Huffman {
    uint16_t count[16];
    uint16_t symbol[320];
    bool build(const uint8_t* lengths, int n) {
        memset(count, 0, sizeof(count));
        for (int i = 0; i < n; ++i) count[lengths[i]]++;
        count[0] = 0;
        int left = 1;  // over-subscribed sets are invalid
        for (int len = 1; len < 16; ++len) {
            left <<= 1;
            left -= count[len];
            if (left < 0) return false;
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; ++len) offs[len + 1] = offs[len] + count[len];
        for (int i = 0; i < n; ++i)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
        return true;
    }
    // Reads one code bit by bit, most significant bit first: the codes of length len are the
    // integers first .. first + count[len] - 1.
    int decode(Bits& b) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; ++len) {
            code |= b.bit();
            const int c = count[len];
            if (code - first < c) return symbol[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

// RFC 1951 section 3.2.5: base values and extra bits of length codes 257..285 and distance codes.
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// Order in which a dynamic block lists the code lengths of the code-length alphabet (3.2.7).
const uint8_t kClOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

bool inflate_codes(Bits& b, const Huffman& lit, const Huffman& dist, Bytes* out, size_t limit) {
    for (;;) {
        const int s = lit.decode(b);
        if (s < 0 || b.over) return false;
        if (s < 256) {
            out->push_back((uint8_t)s);
        } else if (s == 256) {
            return true;
        } else {
            const int li = s - 257;
            if (li >= 29) return false;
            const size_t len = kLenBase[li] + b.bits(kLenExtra[li]);
            const int di = dist.decode(b);
            if (di < 0 || di >= 30) return false;
            const size_t d = kDistBase[di] + b.bits(kDistExtra[di]);
            if (d > out->size() || b.over) return false;
            const size_t start = out->size() - d;
            for (size_t i = 0; i < len; ++i) out->push_back((*out)[start + i]);  // may overlap itself
        }
        if (out->size() > limit) return false;
    }
}

bool inflate(const uint8_t* p, size_t n, Bytes* out, size_t limit) {
    Bits b{p, n};
    int last;
    do {
        last = b.bit();
        const int type = (int)b.bits(2);
        if (b.over) return false;
        if (type == 0) {  // stored
            b.align();
            if (b.pos + 4 > n) return false;
            const uint32_t len = p[b.pos] | p[b.pos + 1] << 8, nlen = p[b.pos + 2] | p[b.pos + 3] << 8;
            b.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || b.pos + len > n) return false;
            out->insert(out->end(), p + b.pos, p + b.pos + len);
            b.pos += len;
        } else if (type == 1) {  // fixed Huffman codes (3.2.6)
            uint8_t l[288], d[30];
            for (int i = 0; i < 144; ++i) l[i] = 8;
            for (int i = 144; i < 256; ++i) l[i] = 9;
            for (int i = 256; i < 280; ++i) l[i] = 7;
            for (int i = 280; i < 288; ++i) l[i] = 8;
            for (int i = 0; i < 30; ++i) d[i] = 5;
            Huffman lit, dist;
            lit.build(l, 288);
            dist.build(d, 30);
            if (!inflate_codes(b, lit, dist, out, limit)) return false;
        } else if (type == 2) {  // dynamic Huffman codes (3.2.7)
            const int hlit = (int)b.bits(5) + 257, hdist = (int)b.bits(5) + 1, hclen = (int)b.bits(4) + 4;
            if (hlit > 286 || hdist > 30) return false;
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; ++i) cl[kClOrder[i]] = (uint8_t)b.bits(3);
            Huffman clh;
            if (!clh.build(cl, 19)) return false;
            uint8_t lens[320] = {0};
            int i = 0;
            while (i < hlit + hdist) {
                const int s = clh.decode(b);
                if (s < 0 || b.over) return false;
                if (s < 16) {
                    lens[i++] = (uint8_t)s;
                    continue;
                }
                int rep, val = 0;
                if (s == 16) {
                    if (i == 0) return false;
                    val = lens[i - 1];
                    rep = 3 + (int)b.bits(2);
                } else if (s == 17) {
                    rep = 3 + (int)b.bits(3);
                } else {
                    rep = 11 + (int)b.bits(7);
                }
                if (i + rep > hlit + hdist) return false;
                while (rep--) lens[i++] = (uint8_t)val;
            }
            if (lens[256] == 0) return false;  // no end-of-block code
            Huffman lit, dist;
            if (!lit.build(lens, hlit) || !dist.build(lens + hlit, hdist)) return false;
            if (!inflate_codes(b, lit, dist, out, limit)) return false;
        } else {
            return false;
        }
    } while (!last);
    return true;
}

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t v = i;
            for (int k = 0; k < 8; ++k) v = (v & 1) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
            table[i] = v;
        }
        init = true;
    }
    c = ~c;
    for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return ~c;
}

uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    for (size_t i = 0; i < n; ++i) {
        a = (a + p[i]) % 65521u;
        b = (b + a) % 65521u;
    }
    return (b << 16) | a;
}

inline uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// ------------------------------------------------------------------------------ PNG

int decode_png(const Bytes& f, Bytes* rgba, int* W, int* H) {
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    if (f.size() < 8 || memcmp(f.data(), sig, 8)) return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: bad signature");
    size_t o = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    Bytes z;
    bool have_trns = false;
    uint16_t key[3] = {0, 0, 0};
    bool seen_end = false;
    while (o + 12 <= f.size()) {
        const uint32_t len = be32(&f[o]);
        if (len > f.size() - o - 12) return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: truncated chunk");
        const uint8_t* type = &f[o + 4];
        const uint8_t* data = &f[o + 8];
        if (crc32(type, 4 + (size_t)len) != be32(data + len)) return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: chunk CRC mismatch");
        if (!memcmp(type, "IHDR", 4)) {
            if (len != 13) return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: bad IHDR");
            w = be32(data);
            h = be32(data + 4);
            depth = data[8];
            ctype = data[9];
            interlace = data[12];
            if (data[10] != 0 || data[11] != 0) return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: unknown compression/filter method");
        } else if (!memcmp(type, "IDAT", 4)) {
            z.insert(z.end(), data, data + len);
        } else if (!memcmp(type, "tRNS", 4)) {
            if (ctype == 0 && len >= 2) {
                key[0] = (uint16_t)(data[0] << 8 | data[1]);
                have_trns = true;
            } else if (ctype == 2 && len >= 6) {
                for (int k = 0; k < 3; ++k) key[k] = (uint16_t)(data[2 * k] << 8 | data[2 * k + 1]);
                have_trns = true;
            }
        } else if (!memcmp(type, "IEND", 4)) {
            seen_end = true;
            break;
        } else if (!(type[0] & 0x20)) {  // critical chunk this decoder does not know (PLTE: palettes)
            return mm::fail(MM_ERR_UNSUPPORTED, "png: unsupported critical chunk %.4s", (const char*)type);
        }
        o += 12 + (size_t)len;
    }
    if (!seen_end || !w || !h) return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: missing IHDR/IEND");
    if (w > 32768 || h > 32768) return mm::fail(MM_ERR_UNSUPPORTED, "png: image larger than 32768");
    int ch;
    switch (ctype) {
        case 0: ch = 1; break;
        case 2: ch = 3; break;
        case 4: ch = 2; break;
        case 6: ch = 4; break;
        default: return mm::fail(MM_ERR_UNSUPPORTED, "png: colour type %d (palette) not supported", ctype);
    }
    if (depth != 8 && depth != 16) return mm::fail(MM_ERR_UNSUPPORTED, "png: bit depth %d not supported", depth);
    if (interlace) return mm::fail(MM_ERR_UNSUPPORTED, "png: interlaced images not supported");
    if (z.size() < 6) return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: no image data");
    const uint8_t cmf = z[0], flg = z[1];
    if ((cmf & 0x0F) != 8 || ((cmf << 8) | flg) % 31 || (flg & 0x20))
        return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: bad zlib header");
    const size_t bpp = (size_t)ch * depth / 8;  // bytes per pixel
    const size_t stride = (size_t)w * bpp;
    const size_t raw_size = (stride + 1) * h;
    Bytes raw;
    raw.reserve(raw_size);
    if (!inflate(z.data() + 2, z.size() - 6, &raw, raw_size) || raw.size() != raw_size)
        return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: corrupt image data");
    if (adler32(raw.data(), raw.size()) != be32(&z[z.size() - 4]))
        return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: Adler-32 mismatch");
    // Reverse the per-row filters (PNG specification section 9) in place.
    Bytes prev(stride, 0), cur(stride);
    rgba->assign((size_t)w * h * 4, 0);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t ft = raw[y * (stride + 1)];
        const uint8_t* s = &raw[y * (stride + 1) + 1];
        for (size_t i = 0; i < stride; ++i) {
            const int a = i >= bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= bpp ? prev[i - bpp] : 0;
            int v = s[i];
            switch (ft) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: {
                    const int pp = a + b - c, pa = abs(pp - a), pb = abs(pp - b), pc = abs(pp - c);
                    v += (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
                    break;
                }
                default: return mm::fail(MM_ERR_INVALID_ARGUMENT, "png: bad filter type %d", ft);
            }
            cur[i] = (uint8_t)v;
        }
        uint8_t* d = &(*rgba)[(size_t)y * w * 4];
        for (uint32_t x = 0; x < w; ++x) {
            uint16_t smp[4];
            for (int k = 0; k < ch; ++k)
                smp[k] = depth == 16 ? (uint16_t)(cur[(x * ch + k) * 2] << 8 | cur[(x * ch + k) * 2 + 1]) : cur[x * ch + k];
            const int hi = depth == 16 ? 8 : 0;
            uint8_t r, g, bl, al = 255;
            if (ch <= 2) {
                r = g = bl = (uint8_t)(smp[0] >> hi);
                if (ch == 2) al = (uint8_t)(smp[1] >> hi);
                if (have_trns && ch == 1 && smp[0] == key[0]) al = 0;
            } else {
                r = (uint8_t)(smp[0] >> hi);
                g = (uint8_t)(smp[1] >> hi);
                bl = (uint8_t)(smp[2] >> hi);
                if (ch == 4) al = (uint8_t)(smp[3] >> hi);
                if (have_trns && ch == 3 && smp[0] == key[0] && smp[1] == key[1] && smp[2] == key[2]) al = 0;
            }
            d[4 * x] = r;
            d[4 * x + 1] = g;
            d[4 * x + 2] = bl;
            d[4 * x + 3] = al;
        }
        prev.swap(cur);
    }
    *W = (int)w;
    *H = (int)h;
    return MM_OK;
}

// ------------------------------------------------------------------------------ TGA

int decode_tga(const Bytes& f, Bytes* rgba, int* W, int* H) {
    if (f.size() < 18) return mm::fail(MM_ERR_INVALID_ARGUMENT, "tga: truncated header");
    const int id_len = f[0], cmap = f[1], type = f[2];
    const int w = f[12] | f[13] << 8, h = f[14] | f[15] << 8, bits = f[16], desc = f[17];
    if (cmap != 0 || (type != 2 && type != 3 && type != 10 && type != 11))
        return mm::fail(MM_ERR_UNSUPPORTED, "tga: image type %d (colour-mapped) not supported", type);
    const bool grey = (type & 3) == 3;
    if (grey ? bits != 8 : (bits != 24 && bits != 32))
        return mm::fail(MM_ERR_UNSUPPORTED, "tga: %d bits per pixel not supported", bits);
    if (w <= 0 || h <= 0) return mm::fail(MM_ERR_INVALID_ARGUMENT, "tga: empty image");
    const int bp = bits / 8;
    const size_t n = (size_t)w * h;
    Bytes px(n * bp);
    size_t o = 18 + (size_t)id_len;
    if (type < 8) {
        if (o + px.size() > f.size()) return mm::fail(MM_ERR_INVALID_ARGUMENT, "tga: truncated pixel data");
        memcpy(px.data(), &f[o], px.size());
    } else {  // run-length packets: count = (c & 0x7F) + 1, a repeated pixel if c & 0x80, else raw pixels
        size_t i = 0;
        while (i < n) {
            if (o >= f.size()) return mm::fail(MM_ERR_INVALID_ARGUMENT, "tga: truncated RLE data");
            const int c = f[o++];
            size_t cnt = (size_t)(c & 0x7F) + 1;
            if (cnt > n - i) cnt = n - i;
            if (c & 0x80) {
                if (o + bp > f.size()) return mm::fail(MM_ERR_INVALID_ARGUMENT, "tga: truncated RLE data");
                for (size_t k = 0; k < cnt; ++k) memcpy(&px[(i + k) * bp], &f[o], bp);
                o += bp;
            } else {
                if (o + cnt * bp > f.size()) return mm::fail(MM_ERR_INVALID_ARGUMENT, "tga: truncated RLE data");
                memcpy(&px[i * bp], &f[o], cnt * bp);
                o += cnt * bp;
            }
            i += cnt;
        }
    }
    const bool top_down = (desc & 0x20) != 0;
    rgba->assign(n * 4, 0);
    for (int y = 0; y < h; ++y) {
        const uint8_t* s = &px[(size_t)(top_down ? y : h - 1 - y) * w * bp];
        uint8_t* d = &(*rgba)[(size_t)y * w * 4];
        for (int x = 0; x < w; ++x, s += bp, d += 4) {
            if (grey) {
                d[0] = d[1] = d[2] = s[0];
                d[3] = 255;
            } else {
                d[0] = s[2];
                d[1] = s[1];
                d[2] = s[0];
                d[3] = bp == 4 ? s[3] : 255;
            }
        }
    }
    *W = w;
    *H = h;
    return MM_OK;
}

int decode_file(const char* path, Bytes* rgba, int* w, int* h) {
    Bytes f;
    if (!path || !read_file(path, &f)) return mm::fail(MM_ERR_INVALID_ARGUMENT, "cannot read %s", path ? path : "(null)");
    if (f.size() >= 8 && f[0] == 0x89 && f[1] == 'P' && f[2] == 'N' && f[3] == 'G') return decode_png(f, rgba, w, h);
    return decode_tga(f, rgba, w, h);
}

}  // namespace

extern "C" int mm_image_decode_file(const char* path, uint8_t** rgba, int* width, int* height) {
    if (!rgba || !width || !height) return mm::fail(MM_ERR_INVALID_ARGUMENT, "decode: null output");
    *rgba = nullptr;
    Bytes px;
    int w = 0, h = 0;
    const int r = decode_file(path, &px, &w, &h);
    if (r) return r;
    uint8_t* out = static_cast<uint8_t*>(malloc(px.size()));
    if (!out) return mm::fail(MM_ERR_OUT_OF_MEMORY, "decode: out of host memory");
    memcpy(out, px.data(), px.size());
    *rgba = out;
    *width = w;
    *height = h;
    return MM_OK;
}

extern "C" int mm_image_free(uint8_t* rgba) {
    free(rgba);
    return MM_OK;
}

extern "C" int mm_texture_load_file(const char* path, int format, mm_texture* out, void* stream) {
    if (!out) return mm::fail(MM_ERR_INVALID_ARGUMENT, "load: null output");
    Bytes px;
    int w = 0, h = 0;
    const int r = decode_file(path, &px, &w, &h);
    if (r) return r;
    return mm_texture_create(px.data(), 0, w, h, 1, 4, format, out, stream);
}

extern "C" int mm_texture_load_slices(const char* prefix, int depth, int format, mm_texture* out, void* stream) {
    if (!out || !prefix || depth <= 0 || depth > 4096) return mm::fail(MM_ERR_INVALID_ARGUMENT, "load: bad arguments");
    Bytes all, px;
    int w0 = 0, h0 = 0;
    for (int i = 0; i < depth; ++i) {
        const std::string path = std::string(prefix) + "(" + std::to_string(i) + ").tga";  // Texture.cpp:511
        int w = 0, h = 0;
        const int r = decode_file(path.c_str(), &px, &w, &h);
        if (r) return r;
        if (i == 0) {
            w0 = w;
            h0 = h;
            all.reserve((size_t)w * h * 4 * depth);
        } else if (w != w0 || h != h0) {
            return mm::fail(MM_ERR_INVALID_ARGUMENT, "load: slice %d is %dx%d, slice 0 is %dx%d", i, w, h, w0, h0);
        }
        all.insert(all.end(), px.begin(), px.end());
    }
    return mm_texture_create(all.data(), 0, w0, h0, depth, 4, format, out, stream);
}
