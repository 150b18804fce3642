// PNG output of the -nogui render loop (SavePNG / SavePNG16 / SavePNG16Alpha,
// src/files.cpp:385-565): signature, IHDR, one IDAT with a zlib stream of stored
// (uncompressed) deflate blocks, IEND. CRC-32 (ISO 3309 polynomial) and Adler-32 are
// computed here, so the writer needs no compression library.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "mbgb.h"
#include "mbgb_internal.h"

namespace {

uint32_t crc_table[256];
bool crc_ready = false;

void crc_init() {
  for (uint32_t n = 0; n < 256; n++) {
    uint32_t c = n;
    for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
    crc_table[n] = c;
  }
  crc_ready = true;
}

uint32_t crc32(const uint8_t *p, size_t n, uint32_t c = 0xFFFFFFFFu) {
  for (size_t i = 0; i < n; i++) c = crc_table[(c ^ p[i]) & 0xFF] ^ (c >> 8);
  return c;
}

void put32(std::vector<uint8_t> &v, uint32_t x) {
  v.push_back((uint8_t)(x >> 24));
  v.push_back((uint8_t)(x >> 16));
  v.push_back((uint8_t)(x >> 8));
  v.push_back((uint8_t)x);
}

bool write_chunk(FILE *f, const char type[4], const std::vector<uint8_t> &data) {
  std::vector<uint8_t> buf;
  put32(buf, (uint32_t)data.size());
  buf.insert(buf.end(), type, type + 4);
  buf.insert(buf.end(), data.begin(), data.end());
  const uint32_t crc = crc32(buf.data() + 4, buf.size() - 4) ^ 0xFFFFFFFFu;
  put32(buf, crc);
  return fwrite(buf.data(), 1, buf.size(), f) == buf.size();
}

}  // namespace

extern "C" mbgb_status mbgb_write_png(const char *path, int32_t width, int32_t height, int32_t bit_depth,
                                      int32_t channels, const void *pixels) {
  if (!path || !pixels || width <= 0 || height <= 0 || (bit_depth != 8 && bit_depth != 16) ||
      (channels != 3 && channels != 4))
    return mbgb::set_error(MBGB_ERR_BAD_PARAM, "mbgb_write_png: bad argument");
  if (!crc_ready) crc_init();
  const size_t bps = (size_t)bit_depth / 8;
  const size_t row = (size_t)width * channels * bps;
  // raw scanlines: filter type 0, samples big-endian
  std::vector<uint8_t> raw;
  raw.reserve((row + 1) * height);
  for (int y = 0; y < height; y++) {
    raw.push_back(0);
    if (bit_depth == 8) {
      const uint8_t *src = (const uint8_t *)pixels + (size_t)y * row;
      raw.insert(raw.end(), src, src + row);
    } else {
      const uint16_t *src = (const uint16_t *)pixels + (size_t)y * width * channels;
      for (size_t i = 0; i < (size_t)width * channels; i++) {
        raw.push_back((uint8_t)(src[i] >> 8));
        raw.push_back((uint8_t)(src[i] & 0xFF));
      }
    }
  }
  // zlib stream: CMF/FLG, stored blocks of at most 65535 bytes, Adler-32
  std::vector<uint8_t> z;
  z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
  z.push_back(0x78);
  z.push_back(0x01);
  size_t pos = 0;
  do {
    const size_t len = std::min<size_t>(65535, raw.size() - pos);
    const bool last = pos + len == raw.size();
    z.push_back(last ? 1 : 0);
    z.push_back((uint8_t)(len & 0xFF));
    z.push_back((uint8_t)(len >> 8));
    z.push_back((uint8_t)(~len & 0xFF));
    z.push_back((uint8_t)((~len >> 8) & 0xFF));
    z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + len);
    pos += len;
  } while (pos < raw.size());
  uint32_t a = 1, b = 0;
  for (uint8_t v : raw) {
    a = (a + v) % 65521u;
    b = (b + a) % 65521u;
  }
  put32(z, (b << 16) | a);
  std::vector<uint8_t> ihdr;
  put32(ihdr, (uint32_t)width);
  put32(ihdr, (uint32_t)height);
  ihdr.push_back((uint8_t)bit_depth);
  ihdr.push_back(channels == 4 ? 6 : 2);   // colour type: RGBA / RGB
  ihdr.push_back(0);                        // deflate
  ihdr.push_back(0);                        // adaptive filtering, filter 0 on every row
  ihdr.push_back(0);                        // no interlace
  FILE *f = fopen(path, "wb");
  if (!f) return mbgb::set_error(MBGB_ERR_IO, std::string("cannot open for writing: ") + path);
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
  bool ok = fwrite(sig, 1, 8, f) == 8;
  ok = ok && write_chunk(f, "IHDR", ihdr);
  ok = ok && write_chunk(f, "IDAT", z);
  ok = ok && write_chunk(f, "IEND", std::vector<uint8_t>());
  ok = (fclose(f) == 0) && ok;
  if (!ok) return mbgb::set_error(MBGB_ERR_IO, std::string("write failed: ") + path);
  return MBGB_OK;
}
