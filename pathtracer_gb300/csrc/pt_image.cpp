// pt_image.cpp -- image files of the C-ABI: pt_load_image / pt_free_image.
//
// Restates the ImageTexture(filename, flip_y, isHDR) constructor
// (src/texture/texture.cpp:3-93), which decodes the file with stb_image
// (vendored as include/external/stb_image.h: stbi_loadf when isHDR,
// stbi_load with 3 requested components otherwise) and stores the pixels as
// texels[x][y]: y = 0 is the image's bottom row, or its top row with flip_y.
// The result here is that array as width*height*3 floats,
// [(y * width + x) * 3 + c], the layout of pt_env_desc and image textures.
//
// Formats (the ones the reference's scenes load):
//   * Radiance RGBE (.hdr): "#?RADIANCE" / "#?RGBE" header with
//     FORMAT=32-bit_rle_rgbe and a "-Y H +X W" resolution line; scanlines
//     flat or in the adaptive run-length encoding; a pixel (r, g, b, e) is
//     c * 2^(e - 136) per channel, 0 when e = 0 (stb's RGBE conversion).
//   * PNG (ISO/IEC 15948, RFC 2083): every colour type and bit depth,
//     non-interlaced or Adam7, zlib / deflate (RFC 1950 / 1951) with stored,
//     fixed and dynamic Huffman blocks; converted to 8-bit RGB as stb does
//     (16-bit samples keep their high byte, grey of depth < 8 is scaled to
//     0..255, grey is replicated, alpha dropped, palette looked up); texels
//     are byte / 255.  With isHDR a PNG is linearised as stbi_loadf does,
//     (byte / 255)^2.2; without it an HDR file is quantised as stbi_load
//     does, (int)(v^(1/2.2) * 255 + 0.5) clamped to 0..255, then / 255.
// Chunk CRCs and the zlib Adler-32 are checked (stb skips both); an
// undecodable file is PT_ERR_INVALID, a missing one PT_ERR_NOT_FOUND.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "pt_host.h"

namespace pt {
namespace {

std::vector<unsigned char> read_file(const char *path, const char *what) {
  FILE *f = std::fopen(path, "rb");
  if (!f) fail(PT_ERR_NOT_FOUND, std::string("cannot open ") + what + " file: " + path);
  std::vector<unsigned char> d;
  unsigned char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) d.insert(d.end(), buf, buf + n);
  std::fclose(f);
  return d;
}

// ---------------------------------------------------------------- Radiance HDR
// Decodes to top-first rows of RGB floats.
void decode_hdr(const std::string &path, const std::vector<unsigned char> &d, std::vector<float> &rgb, int &W,
                int &H) {
  size_t pos = 0;
  auto bad = [&](const char *why) { fail(PT_ERR_INVALID, path + ": " + why); };
  auto line = [&]() {
    std::string s;
    while (pos < d.size() && d[pos] != '\n') s.push_back((char)d[pos++]);
    if (pos >= d.size()) bad("truncated header");
    ++pos;
    if (!s.empty() && s.back() == '\r') s.pop_back();
    return s;
  };
  const std::string magic = line();
  if (magic.rfind("#?RADIANCE", 0) != 0 && magic.rfind("#?RGBE", 0) != 0) bad("not a Radiance HDR file");
  bool rgbe = false;
  for (;;) {
    const std::string s = line();
    if (s.empty()) break;
    if (s == "FORMAT=32-bit_rle_rgbe") rgbe = true;
  }
  if (!rgbe) bad("unsupported FORMAT");
  if (std::sscanf(line().c_str(), "-Y %d +X %d", &H, &W) != 2 || W <= 0 || H <= 0 || W > (1 << 16) ||
      H > (1 << 16))
    bad("unsupported resolution line");
  std::vector<unsigned char> px((size_t)W * 4);
  rgb.assign((size_t)W * H * 3, 0.f);
  auto get = [&]() -> int {
    if (pos >= d.size()) bad("truncated pixels");
    return d[pos++];
  };
  for (int y = 0; y < H; ++y) {
    const int c0 = get(), c1 = get(), c2 = get(), c3 = get();
    if (c0 == 2 && c1 == 2 && !(c2 & 0x80) && W >= 8 && W < 32768) {
      if (((c2 << 8) | c3) != W) bad("scanline width mismatch");
      for (int ch = 0; ch < 4; ++ch)
        for (int x = 0; x < W;) {
          int count = get();
          if (count > 128) {  // a run of one value
            count -= 128;
            const int v = get();
            if (x + count > W) bad("run past the scanline");
            for (int k = 0; k < count; ++k) px[(size_t)(x++) * 4 + ch] = (unsigned char)v;
          } else {            // literal bytes
            if (count == 0 || x + count > W) bad("literal past the scanline");
            for (int k = 0; k < count; ++k) px[(size_t)(x++) * 4 + ch] = (unsigned char)get();
          }
        }
    } else {  // flat RGBE pixels
      px[0] = (unsigned char)c0;
      px[1] = (unsigned char)c1;
      px[2] = (unsigned char)c2;
      px[3] = (unsigned char)c3;
      if (d.size() - pos < (size_t)(W - 1) * 4) bad("truncated pixels");
      std::memcpy(px.data() + 4, d.data() + pos, (size_t)(W - 1) * 4);
      pos += (size_t)(W - 1) * 4;
    }
    float *o = rgb.data() + (size_t)y * W * 3;
    for (int x = 0; x < W; ++x) {
      const unsigned char *p = px.data() + (size_t)x * 4;
      if (!p[3]) continue;
      const float s = std::ldexp(1.0f, (int)p[3] - 136);
      o[3 * x] = p[0] * s;
      o[3 * x + 1] = p[1] * s;
      o[3 * x + 2] = p[2] * s;
    }
  }
}

// ---------------------------------------------------------------- inflate
// RFC 1951.  Huffman codes are decoded through a 10-bit table on the
// least-significant-bit-first stream, with a canonical walk for longer codes.
struct Huffman {
  static constexpr int FAST = 10;
  uint16_t fast[1 << FAST];  // (symbol << 4) | length, 0 = not in the table
  uint16_t count[16];
  uint16_t symbol[288];
};

// Canonical code from per-symbol lengths; false when over-subscribed
// (incomplete sets are allowed: a lone distance code is legal).
bool build_huffman(Huffman &h, const uint8_t *len, int nsym) {
  std::memset(h.count, 0, sizeof h.count);
  for (int s = 0; s < nsym; ++s) h.count[len[s]]++;
  h.count[0] = 0;
  int left = 1;
  for (int l = 1; l < 16; ++l) {
    left = left * 2 - h.count[l];
    if (left < 0) return false;
  }
  uint16_t offs[16];
  offs[1] = 0;
  for (int l = 1; l < 15; ++l) offs[l + 1] = offs[l] + h.count[l];
  for (int s = 0; s < nsym; ++s)
    if (len[s]) h.symbol[offs[len[s]]++] = (uint16_t)s;
  std::memset(h.fast, 0, sizeof h.fast);
  unsigned code = 0;
  int idx = 0;
  for (int l = 1; l <= Huffman::FAST; ++l) {
    for (int k = 0; k < h.count[l]; ++k, ++code, ++idx) {
      unsigned rev = 0;  // codes are sent most significant bit first
      for (int b = 0; b < l; ++b) rev |= ((code >> b) & 1u) << (l - 1 - b);
      for (unsigned f = rev; f < (1u << Huffman::FAST); f += 1u << l) h.fast[f] = (uint16_t)((h.symbol[idx] << 4) | l);
    }
    code <<= 1;
  }
  return true;
}

// the fixed codes of RFC 1951 section 3.2.6
struct FixedCodes {
  Huffman lit, dist;
  FixedCodes() {
    uint8_t l[288];
    for (int s = 0; s < 288; ++s) l[s] = s < 144 ? 8 : s < 256 ? 9 : s < 280 ? 7 : 8;
    build_huffman(lit, l, 288);
    for (int s = 0; s < 30; ++s) l[s] = 5;
    build_huffman(dist, l, 30);
  }
};

struct Inflater {
  const unsigned char *p;
  size_t n, pos = 0;
  uint64_t bits = 0;
  int nbits = 0;
  std::vector<unsigned char> out;
  std::string where;

  [[noreturn]] void bad(const char *why) { fail(PT_ERR_INVALID, where + ": deflate: " + why); }
  void refill() {
    while (nbits <= 56) {
      if (pos < n) bits |= (uint64_t)p[pos] << nbits;
      ++pos;  // reads past the end count as zero bits; checked when used
      nbits += 8;
    }
  }
  unsigned take(int k) {
    if (nbits < k) refill();
    const unsigned v = (unsigned)(bits & ((1ull << k) - 1));
    bits >>= k;
    nbits -= k;
    return v;
  }
  // consumed bits (pos * 8 - nbits) past the input's n * 8
  void check_overrun() {
    if (pos > n && (pos - n) * 8 > (size_t)nbits) bad("input ends inside a block");
  }
  void build(Huffman &h, const uint8_t *len, int nsym) {
    if (!build_huffman(h, len, nsym)) bad("over-subscribed code lengths");
  }

  int decode(const Huffman &h) {
    if (nbits < 16) refill();
    const uint16_t e = h.fast[bits & ((1u << Huffman::FAST) - 1)];
    if (e) {
      bits >>= (e & 15);
      nbits -= (e & 15);
      return e >> 4;
    }
    int code = 0, first = 0, index = 0;
    for (int l = 1; l < 16; ++l) {
      code |= (int)((bits >> (l - 1)) & 1);
      const int c = h.count[l];
      if (code - first < c) {
        bits >>= l;
        nbits -= l;
        return h.symbol[index + code - first];
      }
      index += c;
      first = (first + c) << 1;
      code <<= 1;
    }
    bad("invalid Huffman code");
  }

  void codes(const Huffman &lit, const Huffman &dist) {
    // length and distance bases / extra bits of RFC 1951 section 3.2.5
    static const uint16_t lbase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                       31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
    static const uint8_t lext[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
    static const uint16_t dbase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                       193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
    static const uint8_t dext[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
    for (;;) {
      const int s = decode(lit);
      if (s < 256) {
        out.push_back((unsigned char)s);
        continue;
      }
      if (s == 256) break;
      if (s > 285) bad("invalid length symbol");
      const int len = lbase[s - 257] + (int)take(lext[s - 257]);
      const int ds = decode(dist);
      if (ds > 29) bad("invalid distance symbol");
      const size_t dd = dbase[ds] + take(dext[ds]);
      if (dd > out.size()) bad("distance before the start of the output");
      check_overrun();
      const size_t from = out.size() - dd;
      for (int k = 0; k < len; ++k) out.push_back(out[from + k]);
    }
    check_overrun();
  }

  void run() {
    static const FixedCodes fixed;
    Huffman lit, dist;
    int last;
    do {
      last = (int)take(1);
      const int type = (int)take(2);
      if (type == 0) {  // stored: byte-aligned LEN, ~LEN, bytes
        take(nbits & 7);
        const unsigned len = take(16), nlen = take(16);
        if ((len ^ 0xffffu) != nlen) bad("stored block length check");
        for (unsigned k = 0; k < len; ++k) out.push_back((unsigned char)take(8));
        check_overrun();
      } else if (type == 1) {
        codes(fixed.lit, fixed.dist);
      } else if (type == 2) {
        const int hlit = (int)take(5) + 257, hdist = (int)take(5) + 1, hclen = (int)take(4) + 4;
        static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
        uint8_t cl[19] = {0};
        for (int k = 0; k < hclen; ++k) cl[order[k]] = (uint8_t)take(3);
        Huffman clh;
        build(clh, cl, 19);
        uint8_t lens[320] = {0};
        for (int k = 0; k < hlit + hdist;) {
          const int s = decode(clh);
          int rep = 0;
          uint8_t v = 0;
          if (s < 16) {
            lens[k++] = (uint8_t)s;
            continue;
          } else if (s == 16) {
            if (k == 0) bad("repeat with no previous length");
            v = lens[k - 1];
            rep = 3 + (int)take(2);
          } else if (s == 17) {
            rep = 3 + (int)take(3);
          } else {
            rep = 11 + (int)take(7);
          }
          if (k + rep > hlit + hdist) bad("code lengths past the end");
          while (rep--) lens[k++] = v;
        }
        if (!lens[256]) bad("no end-of-block code");
        build(lit, lens, hlit);
        build(dist, lens + hlit, hdist);
        codes(lit, dist);
      } else {
        bad("invalid block type");
      }
    } while (!last);
  }
};

uint32_t crc32_of(const unsigned char *p, size_t n, uint32_t c = 0xffffffffu) {
  for (size_t i = 0; i < n; ++i) {
    c ^= p[i];
    for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xedb88320u & (0u - (c & 1u)));
  }
  return c;
}

uint32_t be32(const unsigned char *p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }

// ---------------------------------------------------------------- PNG
// Decodes to top-first rows of 8-bit RGB.
void decode_png(const std::string &path, const std::vector<unsigned char> &d, std::vector<unsigned char> &rgb,
                int &W, int &H) {
  auto bad = [&](const std::string &why) { fail(PT_ERR_INVALID, path + ": " + why); };
  static const unsigned char sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  if (d.size() < 8 || std::memcmp(d.data(), sig, 8)) bad("not a PNG file");
  size_t pos = 8;
  int depth = 0, ctype = -1, interlace = 0;
  std::vector<unsigned char> idat, palette;
  bool ended = false;
  while (!ended) {
    if (d.size() - pos < 12) bad("truncated chunk");
    const uint32_t len = be32(&d[pos]);
    if (len > d.size() - pos - 12) bad("truncated chunk");
    const unsigned char *type = &d[pos + 4], *body = &d[pos + 8];
    if (crc32_of(type, len + 4) ^ 0xffffffffu ^ be32(body + len)) bad("chunk CRC mismatch");
    const std::string t((const char *)type, 4);
    if (t == "IHDR") {
      if (len != 13) bad("bad IHDR");
      W = (int)be32(body);
      H = (int)be32(body + 4);
      depth = body[8];
      ctype = body[9];
      interlace = body[12];
      if (W <= 0 || H <= 0 || W > (1 << 16) || H > (1 << 16)) bad("unsupported image size");
      if (body[10] != 0 || body[11] != 0 || interlace > 1) bad("unsupported compression, filter or interlace");
      const bool ok = (ctype == 0 && (depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16)) ||
                      (ctype == 3 && (depth == 1 || depth == 2 || depth == 4 || depth == 8)) ||
                      ((ctype == 2 || ctype == 4 || ctype == 6) && (depth == 8 || depth == 16));
      if (!ok) bad("invalid colour type / bit depth");
    } else if (t == "PLTE") {
      palette.assign(body, body + len);
    } else if (t == "IDAT") {
      idat.insert(idat.end(), body, body + len);
    } else if (t == "IEND") {
      ended = true;
    } else if (!(type[0] & 0x20)) {
      bad("unknown critical chunk " + t);
    }
    pos += 12 + len;
  }
  if (ctype < 0) bad("no IHDR");
  if (ctype == 3 && (palette.empty() || palette.size() % 3)) bad("missing or bad PLTE");
  // zlib stream (RFC 1950): CMF, FLG, deflate data, Adler-32
  if (idat.size() < 6) bad("no image data");
  if ((idat[0] & 15) != 8 || ((idat[0] << 8) | idat[1]) % 31 || (idat[1] & 0x20)) bad("bad zlib header");
  Inflater z;
  z.p = idat.data() + 2;
  z.n = idat.size() - 2;
  z.where = path;
  const int channels = ctype == 0 ? 1 : ctype == 2 ? 3 : ctype == 3 ? 1 : ctype == 4 ? 2 : 4;
  const size_t bits_px = (size_t)channels * depth;
  z.out.reserve(((size_t)W * bits_px + 15) / 8 * H + H);
  z.run();
  {
    // the Adler-32 follows the last block at the next byte boundary
    z.take(z.nbits & 7);
    uint32_t a = 1, b = 0;
    for (unsigned char c : z.out) {
      a = (a + c) % 65521u;
      b = (b + a) % 65521u;
    }
    uint32_t want = 0;
    for (int k = 0; k < 4; ++k) want = want << 8 | z.take(8);
    z.check_overrun();
    if (want != ((b << 16) | a)) bad("zlib Adler-32 mismatch");
  }
  // unfilter each pass (one pass, or the seven of Adam7) into samples
  const int bpp = (int)((bits_px + 7) / 8);  // filter byte distance
  std::vector<uint16_t> samp((size_t)W * H * channels);
  static const int ax0[7] = {0, 4, 0, 2, 0, 1, 0}, ay0[7] = {0, 0, 4, 0, 2, 0, 1};
  static const int adx[7] = {8, 8, 4, 4, 2, 2, 1}, ady[7] = {8, 8, 8, 4, 4, 2, 2};
  size_t in = 0;
  std::vector<unsigned char> prev, cur;
  for (int pass = 0; pass < (interlace ? 7 : 1); ++pass) {
    const int x0 = interlace ? ax0[pass] : 0, y0 = interlace ? ay0[pass] : 0;
    const int dx = interlace ? adx[pass] : 1, dy = interlace ? ady[pass] : 1;
    const int pw = W > x0 ? (W - x0 + dx - 1) / dx : 0, ph = H > y0 ? (H - y0 + dy - 1) / dy : 0;
    if (!pw || !ph) continue;
    const size_t row = ((size_t)pw * bits_px + 7) / 8;
    prev.assign(row, 0);
    cur.resize(row);
    for (int r = 0; r < ph; ++r) {
      if (z.out.size() - in < row + 1) bad("image data too short");
      const int f = z.out[in++];
      const unsigned char *src = z.out.data() + in;
      in += row;
      for (size_t i = 0; i < row; ++i) {
        const int a = i >= (size_t)bpp ? cur[i - bpp] : 0, b = prev[i], c = i >= (size_t)bpp ? prev[i - bpp] : 0;
        int v = 0;
        switch (f) {
        case 0: v = 0; break;
        case 1: v = a; break;
        case 2: v = b; break;
        case 3: v = (a + b) >> 1; break;
        case 4: {  // Paeth predictor
          const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
          v = (pa <= pb && pa <= pc) ? a : (pb <= pc ? b : c);
          break;
        }
        default: bad("invalid filter type");
        }
        cur[i] = (unsigned char)(src[i] + v);
      }
      const int y = y0 + r * dy;
      for (int k = 0; k < pw; ++k) {
        uint16_t *o = samp.data() + ((size_t)y * W + x0 + (size_t)k * dx) * channels;
        for (int ch = 0; ch < channels; ++ch) {
          const size_t s = (size_t)k * channels + ch;
          if (depth == 16) {
            o[ch] = (uint16_t)(cur[2 * s] << 8 | cur[2 * s + 1]);
          } else if (depth == 8) {
            o[ch] = cur[s];
          } else {  // packed from the most significant bit
            const size_t bit = s * depth;
            o[ch] = (uint16_t)((cur[bit >> 3] >> (8 - depth - (bit & 7))) & ((1 << depth) - 1));
          }
        }
      }
      std::swap(prev, cur);
    }
  }
  // to 8-bit RGB
  rgb.resize((size_t)W * H * 3);
  const int grey_scale = depth == 1 ? 255 : depth == 2 ? 0x55 : depth == 4 ? 0x11 : 1;
  for (size_t i = 0; i < (size_t)W * H; ++i) {
    const uint16_t *s = samp.data() + i * channels;
    unsigned char *o = rgb.data() + 3 * i;
    auto to8 = [&](uint16_t v) { return (unsigned char)(depth == 16 ? v >> 8 : v); };
    if (ctype == 3) {
      if ((size_t)s[0] * 3 + 2 >= palette.size()) bad("palette index out of range");
      std::memcpy(o, &palette[(size_t)s[0] * 3], 3);
    } else if (ctype == 0 || ctype == 4) {
      const unsigned char g = depth < 8 ? (unsigned char)(s[0] * grey_scale) : to8(s[0]);
      o[0] = o[1] = o[2] = g;
    } else {
      o[0] = to8(s[0]);
      o[1] = to8(s[1]);
      o[2] = to8(s[2]);
    }
  }
}

// ImageTexture's texels from the file at path.
void load_image(const std::string &path, bool flip_y, bool is_hdr, std::vector<float> &tex, int &W, int &H) {
  const std::vector<unsigned char> d = read_file(path.c_str(), "image");
  std::vector<float> rows;  // top-first RGB
  const bool radiance = d.size() >= 2 && d[0] == '#' && d[1] == '?';
  if (radiance) {
    decode_hdr(path, d, rows, W, H);
    if (!is_hdr)  // stbi_load of an HDR file: v^(1/2.2) * 255 + 0.5, clamped, truncated, then / 255
      for (float &v : rows) {
        float z = std::pow(v, 1.0f / 2.2f) * 255 + 0.5f;
        z = z < 0 ? 0 : z > 255 ? 255 : z;
        v = (float)(int)z / 255.0f;
      }
  } else {
    std::vector<unsigned char> rgb8;
    decode_png(path, d, rgb8, W, H);
    rows.resize(rgb8.size());
    for (size_t i = 0; i < rgb8.size(); ++i)
      rows[i] = is_hdr ? std::pow(rgb8[i] / 255.0f, 2.2f) : rgb8[i] / 255.0f;
  }
  tex.resize(rows.size());
  for (int y = 0; y < H; ++y) {
    const int ty = flip_y ? y : H - 1 - y;  // texels[x][ty] = file row y
    std::memcpy(tex.data() + (size_t)ty * W * 3, rows.data() + (size_t)y * W * 3, sizeof(float) * 3 * W);
  }
}

}  // namespace
}  // namespace pt

using namespace pt;

extern "C" {

int pt_load_image(const char *path, int32_t flip_y, int32_t is_hdr, float **texels, int32_t *width,
                  int32_t *height) {
  if (!path || !texels || !width || !height) return record_error(PT_ERR_INVALID, "pt_load_image: null argument");
  *texels = nullptr;
  try {
    std::vector<float> v;
    int W = 0, H = 0;
    load_image(path, flip_y != 0, is_hdr != 0, v, W, H);
    float *p = static_cast<float *>(std::malloc(v.size() * sizeof(float)));
    if (!p) throw std::bad_alloc();
    std::memcpy(p, v.data(), v.size() * sizeof(float));
    *texels = p;
    *width = W;
    *height = H;
    return PT_OK;
  } catch (const PtError &e) {
    return record_error(e.code, e.what());
  } catch (const std::bad_alloc &) {
    return record_error(PT_ERR_NOMEM, "host out of memory");
  }
}

int pt_free_image(float *texels) {
  std::free(texels);
  return PT_OK;
}

}  // extern "C"
