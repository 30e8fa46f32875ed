/* PNG writer for vkvg_surface_write_to_png: RGBA8, one IDAT with zlib
   "stored" (uncompressed) deflate blocks, CRC-32 and Adler-32 computed here,
   so the library needs no compression dependency.  vkvg itself encodes with
   stb_image_write (src/vkvg_surface.c:384); the decoded pixels are the same. */
#include "host.h"

#include <stdio.h>

/* the CRC-32 table (reflected polynomial 0xEDB88320), built at compile
   time so that concurrent writers share it without initialisation races */
struct Crc32Table {
    uint32_t v[256];
    constexpr Crc32Table() : v() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++)
                c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            v[i] = c;
        }
    }
};
static constexpr Crc32Table crc32_table{};

static uint32_t crc32_update(uint32_t c, const uint8_t *b, size_t n) {
    for (size_t i = 0; i < n; i++)
        c = crc32_table.v[(c ^ b[i]) & 0xFF] ^ (c >> 8);
    return c;
}
static void put_be32(uint8_t *p, uint32_t v) {
    p[0] = (uint8_t)(v >> 24);
    p[1] = (uint8_t)(v >> 16);
    p[2] = (uint8_t)(v >> 8);
    p[3] = (uint8_t)v;
}
static bool write_chunk(FILE *f, const char *type, const uint8_t *data, uint32_t len) {
    uint8_t hdr[8];
    put_be32(hdr, len);
    memcpy(hdr + 4, type, 4);
    uint32_t c = crc32_update(0xFFFFFFFFu, (const uint8_t *)type, 4);
    c          = crc32_update(c, data, len) ^ 0xFFFFFFFFu;
    uint8_t crc[4];
    put_be32(crc, c);
    return fwrite(hdr, 1, 8, f) == 8 && (!len || fwrite(data, 1, len, f) == len) && fwrite(crc, 1, 4, f) == 4;
}

int gb_png_write(const char *path, uint32_t w, uint32_t h, const uint8_t *rgba) {
    size_t               row = 1 + (size_t)w * 4, raw_len = (size_t)h * row;
    std::vector<uint8_t> raw(raw_len);
    for (uint32_t y = 0; y < h; y++) {
        raw[y * row] = 0; /* filter: none */
        memcpy(&raw[y * row + 1], rgba + (size_t)y * w * 4, (size_t)w * 4);
    }
    std::vector<uint8_t> z;
    z.reserve(raw_len + raw_len / 65535 * 5 + 16);
    z.push_back(0x78);
    z.push_back(0x01);
    uint32_t a = 1, b = 0;
    size_t   pos = 0;
    do {
        size_t n    = std::min<size_t>(65535, raw_len - pos);
        bool   last = pos + n == raw_len;
        z.push_back(last ? 1 : 0);
        z.push_back((uint8_t)(n & 0xFF));
        z.push_back((uint8_t)(n >> 8));
        z.push_back((uint8_t)(~n & 0xFF));
        z.push_back((uint8_t)((~n >> 8) & 0xFF));
        z.insert(z.end(), raw.begin() + pos, raw.begin() + pos + n);
        for (size_t i = 0; i < n; i++) {
            a = (a + raw[pos + i]) % 65521u;
            b = (b + a) % 65521u;
        }
        pos += n;
    } while (pos < raw_len);
    uint8_t ad[4];
    put_be32(ad, (b << 16) | a);
    z.insert(z.end(), ad, ad + 4);
    FILE *f = fopen(path, "wb");
    if (!f)
        return 1;
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    uint8_t              ihdr[13];
    put_be32(ihdr, w);
    put_be32(ihdr + 4, h);
    ihdr[8]  = 8; /* bit depth */
    ihdr[9]  = 6; /* RGBA */
    ihdr[10] = ihdr[11] = ihdr[12] = 0;
    bool ok = fwrite(sig, 1, 8, f) == 8 && write_chunk(f, "IHDR", ihdr, 13) &&
              write_chunk(f, "IDAT", z.data(), (uint32_t)z.size()) && write_chunk(f, "IEND", nullptr, 0);
    ok &= fclose(f) == 0;
    return ok ? 0 : 1;
}
