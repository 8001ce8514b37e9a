// PNG and JPEG decoding to RGBA8 (see imagedec.h).
#include "imagedec.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace swr {

// ------------------------------------------------------------------ inflate

namespace {

struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;
    bool bad = false;
    uint32_t get(int need) {
        while (cnt < need) {
            if (pos >= n) {
                bad = true;
                return 0;
            }
            buf |= (uint32_t)p[pos++] << cnt;
            cnt += 8;
        }
        const uint32_t v = buf & ((1u << need) - 1u);
        buf >>= need;
        cnt -= need;
        return v;
    }
};

// Canonical Huffman code: symbols ordered by (length, value); decoding walks
// the lengths one bit at a time.
struct Huff {
    uint16_t count[16] = {};
    uint16_t sym[320] = {};
};

bool huff_build(Huff& h, const uint8_t* len, int n) {
    std::memset(h.count, 0, sizeof(h.count));
    for (int i = 0; i < n; ++i) h.count[len[i]]++;
    h.count[0] = 0;
    int left = 1;
    for (int l = 1; l < 16; ++l) {
        left <<= 1;
        left -= h.count[l];
        if (left < 0) return false;  // over-subscribed
    }
    uint16_t off[16];
    off[1] = 0;
    for (int l = 1; l < 15; ++l) off[l + 1] = (uint16_t)(off[l] + h.count[l]);
    for (int i = 0; i < n; ++i)
        if (len[i]) h.sym[off[len[i]]++] = (uint16_t)i;
    return true;
}

int huff_decode(Bits& b, const Huff& h) {
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
        code |= (int)b.get(1);
        if (b.bad) return -1;
        const int c = h.count[l];
        if (code - c < first) return h.sym[index + (code - first)];
        index += c;
        first = (first + c) << 1;
        code <<= 1;
    }
    return -1;
}

// RFC 1951 length and distance code bases and extra bits.
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(Bits& b, const Huff& lit, const Huff& dist, size_t limit, std::vector<uint8_t>& out,
                   std::string& err) {
    for (;;) {
        const int s = huff_decode(b, lit);
        if (s < 0) {
            err = "deflate: bad literal/length code";
            return false;
        }
        if (s < 256) {
            if (out.size() >= limit) {
                err = "deflate: output larger than expected";
                return false;
            }
            out.push_back((uint8_t)s);
            continue;
        }
        if (s == 256) return true;
        const int li = s - 257;
        if (li >= 29) {
            err = "deflate: bad length code";
            return false;
        }
        const size_t len = kLenBase[li] + b.get(kLenExtra[li]);
        const int ds = huff_decode(b, dist);
        if (ds < 0 || ds >= 30) {
            err = "deflate: bad distance code";
            return false;
        }
        const size_t d = kDistBase[ds] + b.get(kDistExtra[ds]);
        if (b.bad || d > out.size()) {
            err = "deflate: distance beyond output";
            return false;
        }
        if (out.size() + len > limit) {
            err = "deflate: output larger than expected";
            return false;
        }
        const size_t from = out.size() - d;
        for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);
    }
}

}  // namespace

bool zlib_inflate(const uint8_t* src, size_t n, size_t limit, std::vector<uint8_t>& out, std::string& err) {
    if (n < 2 || (src[0] & 0x0F) != 8 || ((src[0] << 8) | src[1]) % 31 != 0 || (src[1] & 0x20)) {
        err = "zlib: bad header";
        return false;
    }
    Bits b{src + 2, n - 2};
    out.clear();
    for (;;) {
        const uint32_t final_ = b.get(1), type = b.get(2);
        if (b.bad) break;
        if (type == 0) {
            b.buf = 0;
            b.cnt = 0;  // skip to the byte boundary
            if (b.pos + 4 > b.n) break;
            const uint32_t len = b.p[b.pos] | (b.p[b.pos + 1] << 8);
            const uint32_t nlen = b.p[b.pos + 2] | (b.p[b.pos + 3] << 8);
            b.pos += 4;
            if ((len ^ 0xFFFFu) != nlen || b.pos + len > b.n || out.size() + len > limit) {
                err = "deflate: bad stored block";
                return false;
            }
            out.insert(out.end(), b.p + b.pos, b.p + b.pos + len);
            b.pos += len;
        } else if (type == 1 || type == 2) {
            Huff lit, dist;
            uint8_t lens[320];
            int nlit, ndist;
            if (type == 1) {
                nlit = 288;
                ndist = 30;
                for (int i = 0; i < 144; ++i) lens[i] = 8;
                for (int i = 144; i < 256; ++i) lens[i] = 9;
                for (int i = 256; i < 280; ++i) lens[i] = 7;
                for (int i = 280; i < 288; ++i) lens[i] = 8;
                for (int i = 0; i < 30; ++i) lens[288 + i] = 5;
            } else {
                nlit = (int)b.get(5) + 257;
                ndist = (int)b.get(5) + 1;
                const int nclen = (int)b.get(4) + 4;
                static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
                uint8_t cl[19] = {};
                for (int i = 0; i < nclen; ++i) cl[order[i]] = (uint8_t)b.get(3);
                Huff ch;
                if (b.bad || nlit > 286 || ndist > 30 || !huff_build(ch, cl, 19)) {
                    err = "deflate: bad dynamic header";
                    return false;
                }
                int i = 0;
                while (i < nlit + ndist) {
                    const int s = huff_decode(b, ch);
                    if (s < 0) {
                        err = "deflate: bad code length code";
                        return false;
                    }
                    if (s < 16) {
                        lens[i++] = (uint8_t)s;
                        continue;
                    }
                    int rep = 0;
                    uint8_t v = 0;
                    if (s == 16) {
                        if (i == 0) {
                            err = "deflate: repeat without a previous length";
                            return false;
                        }
                        v = lens[i - 1];
                        rep = 3 + (int)b.get(2);
                    } else if (s == 17) {
                        rep = 3 + (int)b.get(3);
                    } else {
                        rep = 11 + (int)b.get(7);
                    }
                    if (i + rep > nlit + ndist) {
                        err = "deflate: too many code lengths";
                        return false;
                    }
                    while (rep--) lens[i++] = v;
                }
                if (lens[256] == 0) {
                    err = "deflate: no end-of-block code";
                    return false;
                }
            }
            if (!huff_build(lit, lens, nlit) || !huff_build(dist, lens + nlit, ndist)) {
                err = "deflate: bad code lengths";
                return false;
            }
            if (!inflate_codes(b, lit, dist, limit, out, err)) return false;
        } else {
            err = "deflate: bad block type";
            return false;
        }
        if (final_) return true;
    }
    err = "deflate: truncated stream";
    return false;
}

// ---------------------------------------------------------------------- PNG

namespace {

inline uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

inline uint8_t paeth(int a, int b, int c) {
    const int p = a + b - c;
    const int pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    if (pb <= pc) return (uint8_t)b;
    return (uint8_t)c;
}

// Reverses the per-scanline filters in place (rows of `stride` bytes, each
// preceded by its filter type byte); `bpp` = bytes per complete pixel (>= 1).
bool unfilter(uint8_t* data, uint32_t rows, size_t stride, size_t bpp, std::vector<uint8_t>& out, std::string& err) {
    out.assign((size_t)rows * stride, 0);
    for (uint32_t y = 0; y < rows; ++y) {
        const uint8_t ft = data[(size_t)y * (stride + 1)];
        const uint8_t* in = data + (size_t)y * (stride + 1) + 1;
        uint8_t* cur = out.data() + (size_t)y * stride;
        const uint8_t* prev = y ? cur - stride : nullptr;
        for (size_t x = 0; x < stride; ++x) {
            const int a = x >= bpp ? cur[x - bpp] : 0;
            const int b = prev ? prev[x] : 0;
            const int c = (prev && x >= bpp) ? prev[x - bpp] : 0;
            int v = in[x];
            switch (ft) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: err = "png: bad filter type"; return false;
            }
            cur[x] = (uint8_t)v;
        }
    }
    return true;
}

}  // namespace

bool decode_png(const uint8_t* d, size_t n, uint32_t& w, uint32_t& h, std::vector<uint8_t>& rgba, std::string& err) {
    static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    if (n < 8 || std::memcmp(d, sig, 8) != 0) {
        err = "png: bad signature";
        return false;
    }
    size_t pos = 8;
    uint32_t depth = 0, ctype = 0, interlace = 0;
    bool have_hdr = false;
    std::vector<uint8_t> idat, plte, trns;
    while (pos + 12 <= n) {
        const uint32_t len = be32(d + pos);
        const uint8_t* type = d + pos + 4;
        if (len > n - pos - 12) {
            err = "png: truncated chunk";
            return false;
        }
        const uint8_t* body = d + pos + 8;
        if (!std::memcmp(type, "IHDR", 4) && len >= 13) {
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
            have_hdr = true;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + (size_t)len;
    }
    if (!have_hdr || w == 0 || h == 0 || w > 65536 || h > 65536 || (uint64_t)w * h > (1ull << 28)) {
        err = "png: missing or unsupported header";
        return false;
    }
    int channels;
    switch (ctype) {
        case 0: channels = 1; break;
        case 2: channels = 3; break;
        case 3: channels = 1; break;
        case 4: channels = 2; break;
        case 6: channels = 4; break;
        default: err = "png: bad colour type"; return false;
    }
    const bool depth_ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                          (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                          ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
    if (!depth_ok || interlace > 1 || (ctype == 3 && plte.empty())) {
        err = "png: unsupported bit depth, interlace or missing palette";
        return false;
    }
    const size_t bits_pp = (size_t)channels * depth;
    const size_t bpp = std::max<size_t>(1, bits_pp / 8);
    // Passes: full image, or the seven Adam7 sub-images.
    struct Pass {
        uint32_t x0, y0, dx, dy;
    };
    const Pass full[1] = {{0, 0, 1, 1}};
    const Pass adam7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4}, {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
    const Pass* passes = interlace ? adam7 : full;
    const int npass = interlace ? 7 : 1;
    size_t total = 0;
    for (int p = 0; p < npass; ++p) {
        const uint32_t pw = (w + passes[p].dx - 1 - passes[p].x0) / passes[p].dx;
        const uint32_t ph = (h + passes[p].dy - 1 - passes[p].y0) / passes[p].dy;
        if (w <= passes[p].x0 || h <= passes[p].y0 || pw == 0 || ph == 0) continue;
        total += (size_t)ph * (1 + (pw * bits_pp + 7) / 8);
    }
    std::vector<uint8_t> raw;
    if (!zlib_inflate(idat.data(), idat.size(), total, raw, err)) return false;
    if (raw.size() != total) {
        err = "png: image data size mismatch";
        return false;
    }
    rgba.assign((size_t)w * h * 4, 0);
    const uint32_t maxv = (1u << depth) - 1u;
    size_t off = 0;
    std::vector<uint8_t> un;
    for (int p = 0; p < npass; ++p) {
        const Pass& ps = passes[p];
        if (w <= ps.x0 || h <= ps.y0) continue;
        const uint32_t pw = (w - ps.x0 + ps.dx - 1) / ps.dx, ph = (h - ps.y0 + ps.dy - 1) / ps.dy;
        const size_t stride = (pw * bits_pp + 7) / 8;
        if (!unfilter(raw.data() + off, ph, stride, bpp, un, err)) return false;
        off += (size_t)ph * (stride + 1);
        for (uint32_t y = 0; y < ph; ++y) {
            const uint8_t* row = un.data() + (size_t)y * stride;
            for (uint32_t x = 0; x < pw; ++x) {
                uint32_t s[4] = {0, 0, 0, 0};
                for (int c = 0; c < channels; ++c) {
                    const size_t bit = ((size_t)x * channels + c) * depth;
                    if (depth == 16) {
                        s[c] = (uint32_t)row[bit / 8] << 8 | row[bit / 8 + 1];
                    } else if (depth == 8) {
                        s[c] = row[bit / 8];
                    } else {
                        s[c] = (row[bit / 8] >> (8 - depth - bit % 8)) & maxv;
                    }
                }
                // Samples to 8 bits: low depths scale to the full range,
                // 16-bit rounds (v * 255 / 65535).
                auto to8 = [&](uint32_t v) -> uint8_t {
                    if (depth == 16) return (uint8_t)((v + 128u) / 257u);
                    if (depth == 8) return (uint8_t)v;
                    return (uint8_t)(v * 255u / maxv);
                };
                uint8_t o[4] = {0, 0, 0, 255};
                if (ctype == 3) {
                    if ((size_t)s[0] * 3 + 3 > plte.size()) {
                        err = "png: palette index out of range";
                        return false;
                    }
                    o[0] = plte[s[0] * 3];
                    o[1] = plte[s[0] * 3 + 1];
                    o[2] = plte[s[0] * 3 + 2];
                    o[3] = s[0] < trns.size() ? trns[s[0]] : 255;
                } else if (ctype == 0) {
                    o[0] = o[1] = o[2] = to8(s[0]);
                    if (trns.size() >= 2 && s[0] == ((uint32_t)trns[0] << 8 | trns[1])) o[3] = 0;
                } else if (ctype == 4) {
                    o[0] = o[1] = o[2] = to8(s[0]);
                    o[3] = to8(s[1]);
                } else if (ctype == 2) {
                    o[0] = to8(s[0]);
                    o[1] = to8(s[1]);
                    o[2] = to8(s[2]);
                    if (trns.size() >= 6 && s[0] == ((uint32_t)trns[0] << 8 | trns[1]) &&
                        s[1] == ((uint32_t)trns[2] << 8 | trns[3]) && s[2] == ((uint32_t)trns[4] << 8 | trns[5]))
                        o[3] = 0;
                } else {
                    o[0] = to8(s[0]);
                    o[1] = to8(s[1]);
                    o[2] = to8(s[2]);
                    o[3] = to8(s[3]);
                }
                const size_t px = ((size_t)(ps.y0 + y * ps.dy) * w + (ps.x0 + x * ps.dx)) * 4;
                std::memcpy(&rgba[px], o, 4);
            }
        }
    }
    return true;
}

// --------------------------------------------------------------------- JPEG

namespace {

const uint8_t kZigzag[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                             12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                             35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                             58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

struct JHuff {
    uint8_t vals[256] = {};
    int maxcode[18] = {}, valptr[17] = {}, mincode[17] = {};
    bool present = false;
};

struct JComp {
    int id = 0, h = 1, v = 1, tq = 0, td = 0, ta = 0;
    int bw = 0, bh = 0;         // blocks across / down (padded to whole MCUs)
    std::vector<uint8_t> pix;   // bw*8 x bh*8 samples
    int dc_pred = 0;
};

struct JBits {
    const uint8_t* p;
    size_t n, pos;
    uint32_t buf = 0;
    int cnt = 0;
    bool marker = false;  // a marker was reached: feed zeros
    int bit() {
        if (cnt == 0) {
            uint8_t byte = 0;
            if (!marker && pos < n) {
                byte = p[pos];
                if (byte == 0xFF) {
                    const uint8_t nx = pos + 1 < n ? p[pos + 1] : 0;
                    if (nx == 0x00) {
                        pos += 2;
                    } else {
                        marker = true;
                        byte = 0;
                    }
                } else {
                    ++pos;
                }
            }
            buf = byte;
            cnt = 8;
        }
        --cnt;
        return (int)((buf >> cnt) & 1u);
    }
    int bits(int k) {
        int v = 0;
        for (int i = 0; i < k; ++i) v = (v << 1) | bit();
        return v;
    }
};

void jhuff_build(JHuff& t, const uint8_t counts[16]) {
    int code = 0, k = 0;
    for (int l = 1; l <= 16; ++l) {
        t.valptr[l] = k;
        t.mincode[l] = code;
        code += counts[l - 1];
        k += counts[l - 1];
        t.maxcode[l] = counts[l - 1] ? code - 1 : -1;
        code <<= 1;
    }
    t.maxcode[17] = 0x7FFFFFFF;
    t.present = true;
}

int jhuff_decode(JBits& b, const JHuff& t) {
    int code = 0;
    for (int l = 1; l <= 16; ++l) {
        code = (code << 1) | b.bit();
        if (t.maxcode[l] >= 0 && code <= t.maxcode[l]) return t.vals[t.valptr[l] + code - t.mincode[l]];
    }
    return -1;
}

inline int extend(int v, int s) { return (s && v < (1 << (s - 1))) ? v - (1 << s) + 1 : v; }

// Separable inverse DCT of one dequantized block (JPEG's definition,
// evaluated in float), level shift and clamp.
void idct8x8(const float in[64], uint8_t* out, int stride) {
    static float c[8][8];
    static bool init = false;
    if (!init) {
        for (int x = 0; x < 8; ++x)
            for (int u = 0; u < 8; ++u)
                c[x][u] = (u == 0 ? 0.70710678118654752f : 1.0f) * std::cos((2.0f * x + 1.0f) * u * 3.14159265358979f / 16.0f);
        init = true;
    }
    float tmp[64];
    for (int y = 0; y < 8; ++y)
        for (int x = 0; x < 8; ++x) {
            float s = 0.0f;
            for (int u = 0; u < 8; ++u) s += c[x][u] * in[y * 8 + u];
            tmp[y * 8 + x] = s * 0.5f;
        }
    for (int x = 0; x < 8; ++x)
        for (int y = 0; y < 8; ++y) {
            float s = 0.0f;
            for (int v = 0; v < 8; ++v) s += c[y][v] * tmp[v * 8 + x];
            const float f = std::round(s * 0.5f + 128.0f);
            out[y * stride + x] = (uint8_t)std::min(255.0f, std::max(0.0f, f));
        }
}

}  // namespace

namespace {

// One scan (ITU T.81 B.2.3) into the components' coefficient blocks:
// sequential (every coefficient of each block), or one progressive pass
// (Annex G.1.2: DC first / refinement, AC first / refinement of the band
// Ss..Se at bit Al, with end-of-band runs). One component: its blocks in
// raster order over the component's own size; several: MCU order.
struct JScan {
    std::vector<JComp*> comps;
    int ss = 0, se = 63, ah = 0, al = 0;
    bool progressive = false;
};

bool decode_scan(JBits& b, const JScan& sc, const JHuff* hdc, const JHuff* hac, std::vector<std::vector<int16_t>>& coef,
                 const std::vector<JComp>& all, uint32_t w, uint32_t h, int hmax, int vmax, int mcux, int mcuy,
                 int restart, std::string& err) {
    int eobrun = 0;
    const bool single = sc.comps.size() == 1;
    int units_x = mcux, units_y = mcuy;
    if (single) {
        const JComp& c = *sc.comps[0];
        const uint32_t cw = (w * (uint32_t)c.h + (uint32_t)hmax - 1) / (uint32_t)hmax;
        const uint32_t ch = (h * (uint32_t)c.v + (uint32_t)vmax - 1) / (uint32_t)vmax;
        units_x = (int)((cw + 7) / 8);
        units_y = (int)((ch + 7) / 8);
    }
    auto block = [&](JComp& c, int bx, int by) -> bool {
        const size_t ci = (size_t)(&c - all.data());
        int16_t* k0 = &coef[ci][((size_t)by * c.bw + bx) * 64];
        const int p1 = 1 << sc.al, m1 = -(1 << sc.al);
        if (!sc.progressive || sc.ss == 0) {
            // DC (and, in a sequential scan, the AC coefficients after it).
            if (sc.ah == 0) {
                const int t = jhuff_decode(b, hdc[c.td]);
                if (t < 0 || t > 11) {
                    err = "jpeg: bad DC code";
                    return false;
                }
                c.dc_pred += extend(b.bits(t), t);
                k0[0] = (int16_t)(c.dc_pred * (1 << sc.al));
            } else if (b.bit()) {
                k0[0] = (int16_t)(k0[0] | p1);
            }
            if (sc.progressive) return true;
            for (int k = 1; k < 64;) {
                const int rs = jhuff_decode(b, hac[c.ta]);
                if (rs < 0) {
                    err = "jpeg: bad AC code";
                    return false;
                }
                const int r = rs >> 4, sz = rs & 15;
                if (sz == 0) {
                    if (r != 15) break;  // end of block
                    k += 16;
                    continue;
                }
                k += r;
                if (k > 63) {
                    err = "jpeg: AC run past the block";
                    return false;
                }
                k0[kZigzag[k]] = (int16_t)extend(b.bits(sz), sz);
                ++k;
            }
            return true;
        }
        if (sc.ah == 0) {  // AC first pass
            if (eobrun > 0) {
                --eobrun;
                return true;
            }
            for (int k = sc.ss; k <= sc.se;) {
                const int rs = jhuff_decode(b, hac[c.ta]);
                if (rs < 0) {
                    err = "jpeg: bad AC code";
                    return false;
                }
                const int r = rs >> 4, sz = rs & 15;
                if (sz == 0) {
                    if (r < 15) {  // end-of-band run of 2^r + r bits blocks, this one included
                        eobrun = (1 << r) - 1;
                        if (r) eobrun += b.bits(r);
                        break;
                    }
                    k += 16;
                    continue;
                }
                k += r;
                if (k > sc.se) {
                    err = "jpeg: AC run past the band";
                    return false;
                }
                k0[kZigzag[k]] = (int16_t)(extend(b.bits(sz), sz) * (1 << sc.al));
                ++k;
            }
            return true;
        }
        // AC refinement (G.1.2.3): a correction bit for each coefficient
        // already nonzero, and new coefficients of magnitude 2^Al.
        auto refine = [&](int16_t& v) {
            if (b.bit() && (v & p1) == 0) v = (int16_t)(v + (v >= 0 ? p1 : m1));
        };
        int k = sc.ss;
        if (eobrun == 0) {
            for (; k <= sc.se; ++k) {
                const int rs = jhuff_decode(b, hac[c.ta]);
                if (rs < 0) {
                    err = "jpeg: bad AC code";
                    return false;
                }
                int r = rs >> 4;
                const int sz = rs & 15;
                int val = 0;
                if (sz) {
                    if (sz != 1) {
                        err = "jpeg: bad AC refinement size";
                        return false;
                    }
                    val = b.bit() ? p1 : m1;
                } else if (r != 15) {
                    eobrun = 1 << r;
                    if (r) eobrun += b.bits(r);
                    break;
                }
                // Skip r zero coefficients (refining the nonzero ones passed on
                // the way); a new coefficient lands on the next zero one.
                for (; k <= sc.se; ++k) {
                    int16_t& cv = k0[kZigzag[k]];
                    if (cv != 0) {
                        refine(cv);
                    } else {
                        if (r == 0) break;
                        --r;
                    }
                }
                if (val) {
                    if (k > sc.se) {
                        err = "jpeg: AC refinement past the band";
                        return false;
                    }
                    k0[kZigzag[k]] = (int16_t)val;
                }
            }
        }
        if (eobrun > 0) {
            for (; k <= sc.se; ++k) {
                int16_t& cv = k0[kZigzag[k]];
                if (cv != 0) refine(cv);
            }
            --eobrun;
        }
        return true;
    };
    int todo = restart;
    for (int uy = 0; uy < units_y; ++uy)
        for (int ux = 0; ux < units_x; ++ux) {
            if (restart && todo == 0) {
                // Expect RSTn: realign to the byte after it.
                b.cnt = 0;
                b.marker = false;
                while (b.pos + 1 < b.n && !(b.p[b.pos] == 0xFF && b.p[b.pos + 1] >= 0xD0 && b.p[b.pos + 1] <= 0xD7))
                    ++b.pos;
                b.pos += 2;
                for (JComp* c : sc.comps) c->dc_pred = 0;
                eobrun = 0;
                todo = restart;
            }
            if (single) {
                if (!block(*sc.comps[0], ux, uy)) return false;
            } else {
                for (JComp* c : sc.comps)
                    for (int by = 0; by < c->v; ++by)
                        for (int bx = 0; bx < c->h; ++bx)
                            if (!block(*c, ux * c->h + bx, uy * c->v + by)) return false;
            }
            if (restart) --todo;
        }
    return true;
}

}  // namespace

bool decode_jpeg(const uint8_t* d, size_t n, uint32_t& w, uint32_t& h, std::vector<uint8_t>& rgba,
                 std::string& err) {
    if (n < 4 || d[0] != 0xFF || d[1] != 0xD8) {
        err = "jpeg: bad signature";
        return false;
    }
    uint16_t qt[4][64] = {};
    JHuff hdc[4], hac[4];
    std::vector<JComp> comps;
    std::vector<std::vector<int16_t>> coef;
    int hmax = 1, vmax = 1, restart = 0, mcux = 0, mcuy = 0;
    bool have_frame = false, progressive = false, any_scan = false;
    size_t pos = 2;
    while (pos + 4 <= n) {
        if (d[pos] != 0xFF) {
            err = "jpeg: expected a marker";
            return false;
        }
        const uint8_t m = d[pos + 1];
        pos += 2;
        if (m == 0xD8 || (m >= 0xD0 && m <= 0xD7) || m == 0x01 || m == 0xFF) {
            if (m == 0xFF) --pos;
            continue;
        }
        if (m == 0xD9) break;
        if (pos + 2 > n) break;
        const size_t len = (size_t)d[pos] << 8 | d[pos + 1];
        if (len < 2 || pos + len > n) {
            err = "jpeg: truncated segment";
            return false;
        }
        const uint8_t* s = d + pos + 2;
        const size_t sl = len - 2;
        if (m == 0xDB) {  // DQT
            size_t i = 0;
            while (i < sl) {
                const int pq = s[i] >> 4, tq = s[i] & 3;
                ++i;
                for (int k = 0; k < 64; ++k) {
                    if (i + (pq ? 2 : 1) > sl) {
                        err = "jpeg: truncated DQT";
                        return false;
                    }
                    qt[tq][kZigzag[k]] = pq ? (uint16_t)(s[i] << 8 | s[i + 1]) : s[i];
                    i += pq ? 2 : 1;
                }
            }
        } else if (m == 0xC4) {  // DHT
            size_t i = 0;
            while (i + 17 <= sl) {
                const int tc = s[i] >> 4, th = s[i] & 3;
                uint8_t counts[16];
                int total = 0;
                for (int k = 0; k < 16; ++k) total += counts[k] = s[i + 1 + k];
                i += 17;
                if (total > 256 || i + total > sl) {
                    err = "jpeg: bad DHT";
                    return false;
                }
                JHuff& t = tc ? hac[th] : hdc[th];
                std::memcpy(t.vals, s + i, total);
                jhuff_build(t, counts);
                i += total;
            }
        } else if (m == 0xC0 || m == 0xC1 || m == 0xC2) {  // SOF0 / SOF1 / SOF2 (progressive)
            if (have_frame) {
                err = "jpeg: more than one frame";
                return false;
            }
            if (sl < 6 || s[0] != 8) {
                err = "jpeg: only 8-bit JPEG is supported";
                return false;
            }
            progressive = m == 0xC2;
            h = (uint32_t)(s[1] << 8 | s[2]);
            w = (uint32_t)(s[3] << 8 | s[4]);
            const int nc = s[5];
            if (w == 0 || h == 0 || (nc != 1 && nc != 3) || sl < 6 + 3 * (size_t)nc) {
                err = "jpeg: unsupported frame (grey or YCbCr only)";
                return false;
            }
            comps.resize(nc);
            for (int c = 0; c < nc; ++c) {
                comps[c].id = s[6 + 3 * c];
                comps[c].h = s[7 + 3 * c] >> 4;
                comps[c].v = s[7 + 3 * c] & 15;
                comps[c].tq = s[8 + 3 * c] & 3;
                if (comps[c].h < 1 || comps[c].h > 4 || comps[c].v < 1 || comps[c].v > 4) {
                    err = "jpeg: bad sampling factors";
                    return false;
                }
                hmax = std::max(hmax, comps[c].h);
                vmax = std::max(vmax, comps[c].v);
            }
            mcux = (int)((w + 8 * hmax - 1) / (8 * hmax));
            mcuy = (int)((h + 8 * vmax - 1) / (8 * vmax));
            coef.resize(nc);
            for (int c = 0; c < nc; ++c) {
                comps[c].bw = mcux * comps[c].h;
                comps[c].bh = mcuy * comps[c].v;
                comps[c].pix.assign((size_t)comps[c].bw * 8 * comps[c].bh * 8, 0);
                coef[c].assign((size_t)comps[c].bw * comps[c].bh * 64, 0);
            }
            have_frame = true;
        } else if (m >= 0xC3 && m <= 0xCF && m != 0xC4 && m != 0xC8 && m != 0xCC) {
            err = "jpeg: lossless, hierarchical and arithmetic-coded JPEG are not supported";
            return false;
        } else if (m == 0xDD) {  // DRI
            if (sl >= 2) restart = s[0] << 8 | s[1];
        } else if (m == 0xDA) {  // SOS
            if (!have_frame || sl < 1) {
                err = "jpeg: scan before frame";
                return false;
            }
            const int ns = s[0];
            if (ns < 1 || ns > (int)comps.size() || sl < 1 + 2 * (size_t)ns + 3) {
                err = "jpeg: bad scan header";
                return false;
            }
            JScan sc;
            sc.progressive = progressive;
            for (int k = 0; k < ns; ++k) {
                const int cid = s[1 + 2 * k], td = s[2 + 2 * k] >> 4, ta = s[2 + 2 * k] & 15;
                if (td > 3 || ta > 3) {
                    err = "jpeg: bad Huffman table id";
                    return false;
                }
                JComp* found = nullptr;
                for (JComp& c : comps)
                    if (c.id == cid) found = &c;
                if (!found) {
                    err = "jpeg: scan names an unknown component";
                    return false;
                }
                found->td = td;
                found->ta = ta;
                sc.comps.push_back(found);
            }
            sc.ss = s[1 + 2 * ns];
            sc.se = s[2 + 2 * ns];
            sc.ah = s[3 + 2 * ns] >> 4;
            sc.al = s[3 + 2 * ns] & 15;
            if (progressive) {
                // G.1.1.1.1: a DC scan has Ss = Se = 0; an AC scan one component
                // and 1 <= Ss <= Se <= 63; refinement lowers Al by one.
                const bool dc = sc.ss == 0;
                if ((dc && sc.se != 0) || (!dc && (sc.se < sc.ss || sc.se > 63 || ns != 1)) || sc.al > 13 ||
                    (sc.ah && sc.ah != sc.al + 1)) {
                    err = "jpeg: bad progressive scan parameters";
                    return false;
                }
            } else if (sc.ss != 0 || sc.se != 63 || sc.ah || sc.al) {
                err = "jpeg: bad sequential scan parameters";
                return false;
            }
            const bool needs_dc = !progressive || (sc.ss == 0 && sc.ah == 0);
            const bool needs_ac = !progressive || sc.ss > 0;
            for (JComp* c : sc.comps)
                if ((needs_dc && !hdc[c->td].present) || (needs_ac && !hac[c->ta].present)) {
                    err = "jpeg: missing Huffman table";
                    return false;
                }
            for (JComp* c : sc.comps) c->dc_pred = 0;
            JBits b{d, n, pos + len};
            if (!decode_scan(b, sc, hdc, hac, coef, comps, w, h, hmax, vmax, mcux, mcuy, restart, err)) return false;
            any_scan = true;
            // Continue after the entropy-coded data: the next marker that is
            // not a stuffed byte or a restart marker.
            size_t q = b.pos;
            while (q + 1 < n && !(d[q] == 0xFF && d[q + 1] != 0x00 && !(d[q + 1] >= 0xD0 && d[q + 1] <= 0xD7))) ++q;
            pos = q;
            continue;
        }
        pos += len;
    }
    if (!any_scan) {
        err = "jpeg: no image data";
        return false;
    }
    // Dequantize and inverse-transform every block, then colour.
    for (size_t ci = 0; ci < comps.size(); ++ci) {
        JComp& c = comps[ci];
        for (int by = 0; by < c.bh; ++by)
            for (int bx = 0; bx < c.bw; ++bx) {
                const int16_t* k0 = &coef[ci][((size_t)by * c.bw + bx) * 64];
                float f[64];
                for (int k = 0; k < 64; ++k) f[k] = (float)k0[k] * (float)qt[c.tq][k];
                idct8x8(f, c.pix.data() + (size_t)by * 8 * c.bw * 8 + (size_t)bx * 8, c.bw * 8);
            }
    }
    // Colour: replicate subsampled components, JFIF YCbCr -> RGB.
    rgba.assign((size_t)w * h * 4, 255);
    for (uint32_t y = 0; y < h; ++y)
        for (uint32_t x = 0; x < w; ++x) {
            float v[3];
            for (size_t k = 0; k < comps.size(); ++k) {
                const JComp& c = comps[k];
                const uint32_t sx = x * (uint32_t)c.h / (uint32_t)hmax, sy = y * (uint32_t)c.v / (uint32_t)vmax;
                v[k] = c.pix[(size_t)sy * c.bw * 8 + sx];
            }
            uint8_t* o = &rgba[((size_t)y * w + x) * 4];
            if (comps.size() == 1) {
                o[0] = o[1] = o[2] = (uint8_t)v[0];
            } else {
                const float Y = v[0], cb = v[1] - 128.0f, cr = v[2] - 128.0f;
                const float rgb[3] = {Y + 1.402f * cr, Y - 0.344136f * cb - 0.714136f * cr, Y + 1.772f * cb};
                for (int k = 0; k < 3; ++k) o[k] = (uint8_t)std::min(255.0f, std::max(0.0f, std::round(rgb[k])));
            }
        }
    return true;
}

bool decode_image(const uint8_t* data, size_t n, uint32_t& w, uint32_t& h, std::vector<uint8_t>& rgba,
                  std::string& err) {
    if (n >= 8 && data[0] == 0x89 && data[1] == 'P' && data[2] == 'N' && data[3] == 'G')
        return decode_png(data, n, w, h, rgba, err);
    if (n >= 3 && data[0] == 0xFF && data[1] == 0xD8) return decode_jpeg(data, n, w, h, rgba, err);
    err = "unsupported image format (PNG and JPEG are decoded)";
    return false;
}

}  // namespace swr
