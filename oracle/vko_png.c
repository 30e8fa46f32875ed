/* vko_png.c - minimal PNG writer for the oracle (RGBA8, zlib "stored"
   blocks, no compression).  Test infrastructure only. */
#include "vko_internal.h"

#include <stdio.h>

static uint32_t crc_table[256];
static int      crc_ready = 0;
static void     crc_init(void) {
    for (uint32_t n = 0; n < 256; n++) {
        uint32_t c = n;
        for (int k = 0; k < 8; k++)
            c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
        crc_table[n] = c;
    }
    crc_ready = 1;
}
static uint32_t crc_update(uint32_t c, const uint8_t *b, size_t n) {
    for (size_t i = 0; i < n; i++)
        c = crc_table[(c ^ b[i]) & 0xFF] ^ (c >> 8);
    return c;
}
static void be32(uint8_t *p, uint32_t v) {
    p[0] = (uint8_t)(v >> 24);
    p[1] = (uint8_t)(v >> 16);
    p[2] = (uint8_t)(v >> 8);
    p[3] = (uint8_t)v;
}
static int chunk(FILE *f, const char *type, const uint8_t *data, uint32_t len) {
    uint8_t hdr[8];
    be32(hdr, len);
    memcpy(hdr + 4, type, 4);
    uint32_t c = crc_update(0xFFFFFFFFu, (const uint8_t *)type, 4);
    c          = crc_update(c, data, len) ^ 0xFFFFFFFFu;
    uint8_t tail[4];
    be32(tail, c);
    return fwrite(hdr, 1, 8, f) != 8 || (len && fwrite(data, 1, len, f) != len) || fwrite(tail, 1, 4, f) != 4;
}
int vko_png_write(const char *path, uint32_t w, uint32_t h, const uint8_t *rgba) {
    if (!crc_ready)
        crc_init();
    size_t   raw_len = (size_t)h * (1 + (size_t)w * 4);
    size_t   nblk    = raw_len / 65535 + 1;
    size_t   zlen    = 2 + raw_len + nblk * 5 + 4;
    uint8_t *z       = (uint8_t *)malloc(zlen);
    uint8_t *raw     = (uint8_t *)malloc(raw_len);
    if (!z || !raw) {
        free(z);
        free(raw);
        return 1;
    }
    for (uint32_t y = 0; y < h; y++) {
        raw[(size_t)y * (1 + w * 4)] = 0;
        memcpy(raw + (size_t)y * (1 + w * 4) + 1, rgba + (size_t)y * w * 4, (size_t)w * 4);
    }
    size_t o = 0;
    z[o++]   = 0x78;
    z[o++]   = 0x01;
    uint32_t a = 1, b = 0;
    size_t   pos = 0;
    do {
        size_t n    = raw_len - pos > 65535 ? 65535 : raw_len - pos;
        int    last = pos + n == raw_len;
        z[o++]      = (uint8_t)last;
        z[o++]      = (uint8_t)(n & 0xFF);
        z[o++]      = (uint8_t)(n >> 8);
        z[o++]      = (uint8_t)(~n & 0xFF);
        z[o++]      = (uint8_t)((~n >> 8) & 0xFF);
        memcpy(z + o, raw + pos, n);
        for (size_t i = 0; i < n; i++) {
            a = (a + raw[pos + i]) % 65521u;
            b = (b + a) % 65521u;
        }
        o += n;
        pos += n;
    } while (pos < raw_len);
    be32(z + o, (b << 16) | a);
    o += 4;
    FILE *f = fopen(path, "wb");
    int   err = !f;
    if (f) {
        static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
        uint8_t              ihdr[13];
        be32(ihdr, w);
        be32(ihdr + 4, h);
        ihdr[8]  = 8;
        ihdr[9]  = 6;
        ihdr[10] = 0;
        ihdr[11] = 0;
        ihdr[12] = 0;
        err |= fwrite(sig, 1, 8, f) != 8;
        err |= chunk(f, "IHDR", ihdr, 13);
        err |= chunk(f, "IDAT", z, (uint32_t)o);
        err |= chunk(f, "IEND", NULL, 0);
        err |= fclose(f) != 0;
    }
    free(z);
    free(raw);
    return err;
}
