// PNG and Radiance RGBE decoding for textures (see image_io.h).
//
// PNG: chunks (IHDR, PLTE, tRNS, IDAT, IEND), the zlib stream of the
// concatenated IDAT data inflated per RFC 1950 / 1951 (stored, fixed- and
// dynamic-Huffman blocks), the five scanline filters (none, sub, up,
// average, Paeth) per pass, Adam7 interlacing, and the sample conversion
// to 8-bit channels described in image_io.h.
// RGBE: the "#?RADIANCE" / "#?RGBE" header, "-Y h +X w" resolution, flat
// or new-style run-length scanlines.
#include "image_io.h"

#include <cmath>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>

namespace cpppt_gb300 {
namespace {

[[noreturn]] void bad(const std::string& what) { throw std::runtime_error("image: " + what); }

// ---------------------------------------------------------------------------
// Inflate (RFC 1951)
// ---------------------------------------------------------------------------
struct BitReader {
    const uint8_t* p;
    size_t n, pos = 0;  // byte position
    uint32_t bitbuf = 0;
    int bitcnt = 0;
    uint32_t bits(int k) {  // k <= 24, LSB first
        while (bitcnt < k) {
            if (pos >= n) bad("truncated deflate stream");
            bitbuf |= (uint32_t)p[pos++] << bitcnt;
            bitcnt += 8;
        }
        const uint32_t v = bitbuf & ((1u << k) - 1u);
        bitbuf >>= k;
        bitcnt -= k;
        return v;
    }
    void align() {
        bitbuf = 0;
        bitcnt = 0;
    }
};

// Canonical Huffman code: counts per length, symbols ordered by code.
struct Huffman {
    uint16_t count[16] = {};
    std::vector<uint16_t> symbol;
    void build(const uint8_t* lengths, int n) {
        std::memset(count, 0, sizeof(count));
        for (int i = 0; i < n; i++) count[lengths[i]]++;
        count[0] = 0;
        int left = 1;
        for (int len = 1; len < 16; len++) {
            left <<= 1;
            left -= count[len];
            if (left < 0) bad("over-subscribed Huffman code");
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; len++) offs[len + 1] = (uint16_t)(offs[len] + count[len]);
        symbol.assign(n, 0);
        for (int i = 0; i < n; i++)
            if (lengths[i]) symbol[offs[lengths[i]]++] = (uint16_t)i;
    }
    int decode(BitReader& br) const {
        int code = 0, first = 0, index = 0;
        for (int len = 1; len < 16; len++) {
            code |= (int)br.bits(1);
            const int c = count[len];
            if (code - c < first) return symbol[index + (code - first)];
            index += c;
            first += c;
            first <<= 1;
            code <<= 1;
        }
        bad("invalid Huffman code");
    }
};

// Length and distance codes (RFC 1951, 3.2.5)
const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void inflate_block(BitReader& br, const Huffman& lit, const Huffman& dist, std::vector<uint8_t>& out) {
    for (;;) {
        const int sym = lit.decode(br);
        if (sym < 256) {
            out.push_back((uint8_t)sym);
        } else if (sym == 256) {
            return;
        } else {
            const int li = sym - 257;
            if (li >= 29) bad("bad length code");
            const int len = kLenBase[li] + (int)br.bits(kLenExtra[li]);
            const int di = dist.decode(br);
            if (di >= 30) bad("bad distance code");
            const size_t d = kDistBase[di] + br.bits(kDistExtra[di]);
            if (d > out.size()) bad("distance beyond the output");
            const size_t from = out.size() - d;
            for (int k = 0; k < len; k++) out.push_back(out[from + k]);
        }
    }
}

std::vector<uint8_t> zlib_inflate(const uint8_t* p, size_t n, size_t expect) {
    if (n < 2) bad("short zlib stream");
    const int cmf = p[0], flg = p[1];
    if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0) bad("not a deflate zlib stream");
    if (flg & 32) bad("zlib preset dictionary");
    BitReader br{p + 2, n - 2};
    std::vector<uint8_t> out;
    out.reserve(expect);
    Huffman flit, fdist;
    bool fixed_built = false;
    int last = 0;
    while (!last) {
        last = (int)br.bits(1);
        const int type = (int)br.bits(2);
        if (type == 0) {  // stored
            br.align();
            if (br.pos + 4 > br.n) bad("truncated stored block");
            const int len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
            const int nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
            if ((len ^ 0xffff) != nlen) bad("stored block length check");
            br.pos += 4;
            if (br.pos + len > br.n) bad("truncated stored block");
            out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
            br.pos += len;
        } else if (type == 1) {  // fixed Huffman codes (3.2.6)
            if (!fixed_built) {
                uint8_t l[288];
                for (int i = 0; i < 144; i++) l[i] = 8;
                for (int i = 144; i < 256; i++) l[i] = 9;
                for (int i = 256; i < 280; i++) l[i] = 7;
                for (int i = 280; i < 288; i++) l[i] = 8;
                flit.build(l, 288);
                uint8_t d[30];
                for (int i = 0; i < 30; i++) d[i] = 5;
                fdist.build(d, 30);
                fixed_built = true;
            }
            inflate_block(br, flit, fdist, out);
        } else if (type == 2) {  // dynamic Huffman codes (3.2.7)
            const int hlit = (int)br.bits(5) + 257, hdist = (int)br.bits(5) + 1, hclen = (int)br.bits(4) + 4;
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {};
            for (int i = 0; i < hclen; i++) cl[order[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            clh.build(cl, 19);
            uint8_t lens[288 + 32] = {};
            int i = 0;
            while (i < hlit + hdist) {
                const int sym = clh.decode(br);
                if (sym < 16) {
                    lens[i++] = (uint8_t)sym;
                } else {
                    int rep, val = 0;
                    if (sym == 16) {
                        if (i == 0) bad("repeat without a previous length");
                        val = lens[i - 1];
                        rep = 3 + (int)br.bits(2);
                    } else if (sym == 17) {
                        rep = 3 + (int)br.bits(3);
                    } else {
                        rep = 11 + (int)br.bits(7);
                    }
                    if (i + rep > hlit + hdist) bad("code lengths overflow");
                    while (rep--) lens[i++] = (uint8_t)val;
                }
            }
            Huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            inflate_block(br, lit, dist, out);
        } else {
            bad("reserved deflate block type");
        }
    }
    return out;
}

// ---------------------------------------------------------------------------
// PNG
// ---------------------------------------------------------------------------
uint32_t be32(const uint8_t* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

int paeth(int a, int b, int c) {
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

// Reverses the filters of one (sub)image of w x h pixels in place; raw
// holds h rows of 1 + stride bytes, rows receives h x stride bytes.
void unfilter(const uint8_t* raw, int w, int h, int bits_pp, std::vector<uint8_t>& rows, size_t& stride) {
    stride = ((size_t)w * bits_pp + 7) / 8;
    const int bpp = std::max(1, bits_pp / 8);
    rows.assign(stride * h, 0);
    for (int y = 0; y < h; y++) {
        const uint8_t* in = raw + (size_t)y * (stride + 1);
        const int ft = in[0];
        in++;
        uint8_t* cur = rows.data() + (size_t)y * stride;
        const uint8_t* prev = y > 0 ? cur - stride : nullptr;
        for (size_t x = 0; x < stride; x++) {
            const int a = x >= (size_t)bpp ? cur[x - bpp] : 0;
            const int b = prev ? prev[x] : 0;
            const int c = (prev && x >= (size_t)bpp) ? prev[x - bpp] : 0;
            int v = in[x];
            switch (ft) {
                case 0: break;
                case 1: v += a; break;
                case 2: v += b; break;
                case 3: v += (a + b) >> 1; break;
                case 4: v += paeth(a, b, c); break;
                default: bad("unknown PNG filter type");
            }
            cur[x] = (uint8_t)v;
        }
    }
}

}  // namespace

DecodedImage decode_png(const uint8_t* d, size_t n) {
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (n < 8 || std::memcmp(d, sig, 8) != 0) bad("not a PNG file");
    size_t pos = 8;
    int w = 0, h = 0, depth = 0, ctype = -1, interlace = 0;
    std::vector<uint8_t> idat, plte, trns;
    bool have_ihdr = false, have_iend = false;
    while (pos + 8 <= n && !have_iend) {
        const uint32_t len = be32(d + pos);
        const uint8_t* type = d + pos + 4;
        if (pos + 12 + (size_t)len > n) bad("truncated PNG chunk");
        const uint8_t* body = d + pos + 8;
        if (!std::memcmp(type, "IHDR", 4)) {
            if (len != 13) bad("bad IHDR");
            w = (int)be32(body);
            h = (int)be32(body + 4);
            depth = body[8];
            ctype = body[9];
            if (body[10] != 0 || body[11] != 0) bad("unknown PNG compression or filter method");
            interlace = body[12];
            have_ihdr = true;
        } else if (!std::memcmp(type, "PLTE", 4)) {
            plte.assign(body, body + len);
        } else if (!std::memcmp(type, "tRNS", 4)) {
            trns.assign(body, body + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            have_iend = true;
        } else if (!(type[0] & 32)) {
            bad("unknown critical PNG chunk");
        }
        pos += 12 + (size_t)len;
    }
    if (!have_ihdr || idat.empty()) bad("PNG without IHDR or IDAT");
    if (w <= 0 || h <= 0 || w > (1 << 24) || h > (1 << 24) || (long long)w * h > (1ll << 28)) bad("PNG size");
    int chans;
    switch (ctype) {
        case 0: chans = 1; break;
        case 2: chans = 3; break;
        case 3: chans = 1; break;
        case 4: chans = 2; break;
        case 6: chans = 4; break;
        default: bad("unknown PNG colour type");
    }
    const bool depth_ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                          (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                          ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
    if (!depth_ok) bad("bad PNG bit depth for its colour type");
    if (interlace > 1) bad("unknown PNG interlace method");
    if (ctype == 3 && (plte.empty() || plte.size() % 3)) bad("PNG palette missing");
    const int bits_pp = chans * depth;
    // raw (filtered) size of all passes
    static const int ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
    static const int adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
    const int passes = interlace ? 7 : 1;
    auto pass_dims = [&](int p, int& pw, int& ph) {
        if (!interlace) { pw = w; ph = h; return; }
        pw = (w - ax0[p] + adx[p] - 1) / adx[p];
        ph = (h - ay0[p] + ady[p] - 1) / ady[p];
        if (w <= ax0[p]) pw = 0;
        if (h <= ay0[p]) ph = 0;
    };
    size_t expect = 0;
    for (int p = 0; p < passes; p++) {
        int pw, ph;
        pass_dims(p, pw, ph);
        if (pw > 0 && ph > 0) expect += (size_t)ph * (1 + ((size_t)pw * bits_pp + 7) / 8);
    }
    const std::vector<uint8_t> raw = zlib_inflate(idat.data(), idat.size(), expect);
    if (raw.size() < expect) bad("PNG image data too short");
    // samples of the whole image: chans samples per pixel, 16-bit kept whole for now
    std::vector<uint16_t> samp((size_t)w * h * chans);
    size_t off = 0;
    for (int p = 0; p < passes; p++) {
        int pw, ph;
        pass_dims(p, pw, ph);
        if (pw <= 0 || ph <= 0) continue;
        std::vector<uint8_t> rows;
        size_t stride;
        unfilter(raw.data() + off, pw, ph, bits_pp, rows, stride);
        off += (size_t)ph * (stride + 1);
        for (int y = 0; y < ph; y++) {
            const uint8_t* r = rows.data() + (size_t)y * stride;
            const int iy = interlace ? ay0[p] + y * ady[p] : y;
            for (int x = 0; x < pw; x++) {
                const int ix = interlace ? ax0[p] + x * adx[p] : x;
                uint16_t* o = samp.data() + ((size_t)iy * w + ix) * chans;
                for (int c = 0; c < chans; c++) {
                    const size_t s = (size_t)x * chans + c;  // sample index in the row
                    uint16_t v;
                    if (depth == 16) v = (uint16_t)((r[2 * s] << 8) | r[2 * s + 1]);
                    else if (depth == 8) v = r[s];
                    else {
                        const size_t bit = s * depth;
                        v = (uint16_t)((r[bit >> 3] >> (8 - depth - (bit & 7))) & ((1 << depth) - 1));
                    }
                    o[c] = v;
                }
            }
        }
    }
    DecodedImage im;
    im.w = w;
    im.h = h;
    if (ctype == 3) {  // palette -> RGB, RGBA where tRNS gives alpha
        const bool alpha = !trns.empty();
        im.n = alpha ? 4 : 3;
        im.u8.resize((size_t)w * h * im.n);
        const size_t np = plte.size() / 3;
        for (size_t i = 0; i < (size_t)w * h; i++) {
            const size_t k = samp[i];
            if (k >= np) bad("PNG palette index out of range");
            uint8_t* o = im.u8.data() + i * im.n;
            o[0] = plte[3 * k];
            o[1] = plte[3 * k + 1];
            o[2] = plte[3 * k + 2];
            if (alpha) o[3] = k < trns.size() ? trns[k] : 255;
        }
        return im;
    }
    im.n = chans;
    im.u8.resize(samp.size());
    static const int scale[9] = {0, 0xff, 0x55, 0, 0x11, 0, 0, 0, 0x01};
    for (size_t i = 0; i < samp.size(); i++)
        im.u8[i] = depth == 16 ? (uint8_t)(samp[i] >> 8) : (uint8_t)(samp[i] * scale[depth]);
    return im;
}

DecodedImage decode_rgbe(const uint8_t* d, size_t n) {
    size_t pos = 0;
    auto line = [&]() {
        std::string s;
        while (pos < n && d[pos] != '\n') s.push_back((char)d[pos++]);
        if (pos >= n) bad("truncated RGBE header");
        pos++;
        return s;
    };
    const std::string magic = line();
    if (magic != "#?RADIANCE" && magic != "#?RGBE") bad("not a Radiance RGBE file");
    bool fmt = false;
    for (;;) {
        const std::string s = line();
        if (s.empty()) break;
        if (s == "FORMAT=32-bit_rle_rgbe") fmt = true;
    }
    if (!fmt) bad("unsupported RGBE format");
    const std::string res = line();
    int h = 0, w = 0;
    if (std::sscanf(res.c_str(), "-Y %d +X %d", &h, &w) != 2 || w <= 0 || h <= 0 || (long long)w * h > (1ll << 28))
        bad("unsupported RGBE resolution line");
    DecodedImage im;
    im.w = w;
    im.h = h;
    im.n = 3;
    im.hdr = true;
    im.f.resize((size_t)w * h * 3);
    std::vector<uint8_t> scan((size_t)w * 4);
    auto put = [&](int y, int x, const uint8_t* e) {
        float* o = im.f.data() + ((size_t)y * w + x) * 3;
        if (e[3] == 0) {
            o[0] = o[1] = o[2] = 0.0f;
            return;
        }
        const float f = std::ldexp(1.0f, (int)e[3] - 136);
        o[0] = e[0] * f;
        o[1] = e[1] * f;
        o[2] = e[2] * f;
    };
    for (int y = 0; y < h; y++) {
        const bool rle = w >= 8 && w < 32768 && pos + 4 <= n && d[pos] == 2 && d[pos + 1] == 2 && !(d[pos + 2] & 0x80);
        if (!rle) {  // flat scanlines (the rest of the file is flat)
            for (int yy = y; yy < h; yy++)
                for (int x = 0; x < w; x++) {
                    if (pos + 4 > n) bad("truncated RGBE data");
                    put(yy, x, d + pos);
                    pos += 4;
                }
            break;
        }
        if (((d[pos + 2] << 8) | d[pos + 3]) != w) bad("RGBE scanline width mismatch");
        pos += 4;
        for (int c = 0; c < 4; c++) {
            int x = 0;
            while (x < w) {
                if (pos >= n) bad("truncated RGBE data");
                int count = d[pos++];
                if (count > 128) {
                    count -= 128;
                    if (pos >= n || x + count > w) bad("bad RGBE run");
                    const uint8_t v = d[pos++];
                    for (int k = 0; k < count; k++) scan[(size_t)(x++) * 4 + c] = v;
                } else {
                    if (count == 0 || x + count > w || pos + count > n) bad("bad RGBE dump");
                    for (int k = 0; k < count; k++) scan[(size_t)(x++) * 4 + c] = d[pos++];
                }
            }
        }
        for (int x = 0; x < w; x++) put(y, x, scan.data() + (size_t)x * 4);
    }
    return im;
}

DecodedImage decode_image_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) bad("cannot open " + path);
    const std::vector<uint8_t> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (data.size() >= 8 && data[0] == 137 && data[1] == 'P' && data[2] == 'N' && data[3] == 'G') {
        return decode_png(data.data(), data.size());
    }
    if (data.size() >= 2 && data[0] == '#' && data[1] == '?') return decode_rgbe(data.data(), data.size());
    bad("unsupported image format (PNG and Radiance .hdr are read): " + path);
}

float srgb_to_linear_ref(float a) {
    if ((double)a > 0.04045) return powf((float)(((double)a + 0.055) / 1.055), 2.4f);
    return (float)((double)a / 12.92);
}

void texture_pixels(const DecodedImage& im, bool rgb, bool srgb, std::vector<float>& out) {
    const size_t np = (size_t)im.w * im.h;
    const int oc = rgb ? 3 : 1;
    out.resize(np * oc);
    for (size_t i = 0; i < np; i++) {
        for (int c = 0; c < oc; c++) {
            const int src = (rgb && im.n >= 3) ? c : 0;  // Image<Vec3> of a grey file replicates channel 0
            float v;
            if (im.hdr) v = im.f[i * im.n + src];
            else v = (float)((double)(float)im.u8[i * im.n + src] / 255.0);  // char2float (rgb_image.h:19-21)
            out[i * oc + c] = srgb ? srgb_to_linear_ref(v) : v;
        }
    }
}

}  // namespace cpppt_gb300
