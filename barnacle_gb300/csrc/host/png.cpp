// bn_image_write_png: an RGBA8 image as PNG (what Film.Save, Base/Film.fs:55-66, has ImageSharp
// write).  The zlib stream uses stored (uncompressed) deflate blocks, so the encoder needs no
// compression library: signature, IHDR (8-bit RGBA), IDAT (filter byte 0 per row), IEND, with
// the CRC-32 of every chunk and the Adler-32 of the image data.
#include <cstdint>
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "../../../include/barnacle_gpu.h"

int bnh_host_fail(int code, const std::string& msg);

namespace {

uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
  static uint32_t table[256];
  static bool init = false;
  if (!init) {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xedb88320u ^ (c >> 1) : c >> 1;
      table[i] = c;
    }
    init = true;
  }
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
  return crc;
}

void put32(std::vector<uint8_t>& v, uint32_t x) {
  v.push_back(static_cast<uint8_t>(x >> 24));
  v.push_back(static_cast<uint8_t>(x >> 16));
  v.push_back(static_cast<uint8_t>(x >> 8));
  v.push_back(static_cast<uint8_t>(x));
}

void chunk(std::vector<uint8_t>& out, const char* type, const std::vector<uint8_t>& data) {
  put32(out, static_cast<uint32_t>(data.size()));
  const size_t start = out.size();
  out.insert(out.end(), type, type + 4);
  out.insert(out.end(), data.begin(), data.end());
  const uint32_t crc = crc32_update(0xffffffffu, out.data() + start, out.size() - start) ^ 0xffffffffu;
  put32(out, crc);
}

}  // namespace

extern "C" int bn_image_write_png(const char* path, const uint8_t* rgba, int32_t width, int32_t height) {
  if (!path || !rgba || width <= 0 || height <= 0) return bnh_host_fail(BN_ERR_INVALID_ARG, "bn_image_write_png: bad arguments");
  const size_t row = static_cast<size_t>(width) * 4 + 1;
  std::vector<uint8_t> raw;
  raw.reserve(row * height);
  for (int y = 0; y < height; ++y) {
    raw.push_back(0);  // filter: none
    const uint8_t* r = rgba + static_cast<size_t>(y) * width * 4;
    raw.insert(raw.end(), r, r + static_cast<size_t>(width) * 4);
  }
  std::vector<uint8_t> z = {0x78, 0x01};  // deflate, 32 K window, no preset dictionary
  for (size_t off = 0; off < raw.size() || off == 0;) {
    const size_t n = std::min<size_t>(65535, raw.size() - off);
    const bool last = off + n >= raw.size();
    z.push_back(last ? 1 : 0);  // BFINAL, BTYPE = 00 (stored)
    z.push_back(static_cast<uint8_t>(n));
    z.push_back(static_cast<uint8_t>(n >> 8));
    z.push_back(static_cast<uint8_t>(~n));
    z.push_back(static_cast<uint8_t>(~n >> 8));
    z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
    off += n;
    if (last) break;
  }
  uint32_t a = 1, b = 0;  // Adler-32
  for (uint8_t c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  put32(z, (b << 16) | a);
  std::vector<uint8_t> out = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
  std::vector<uint8_t> ihdr;
  put32(ihdr, static_cast<uint32_t>(width));
  put32(ihdr, static_cast<uint32_t>(height));
  ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit, RGBA, deflate, adaptive filters, no interlace
  chunk(out, "IHDR", ihdr);
  chunk(out, "IDAT", z);
  chunk(out, "IEND", {});
  FILE* f = std::fopen(path, "wb");
  if (!f) return bnh_host_fail(BN_ERR_INVALID_ARG, std::string("cannot write ") + path);
  const size_t w = std::fwrite(out.data(), 1, out.size(), f);
  const bool ok = std::fclose(f) == 0 && w == out.size();
  return ok ? BN_OK : bnh_host_fail(BN_ERR_INVALID_ARG, std::string("short write to ") + path);
}
