/*
 * ORACLE — test infrastructure only (see oracle.h).
 *
 * Restatement of the reference's DSD packers, src/dop.c:114-184:
 *   DoP 24-bit little-endian frames [bits 7..0, bits 15..8, marker] where the
 *   16 DSD bits of a frame are taken MSB first and the marker alternates
 *   0x05 / 0xFA starting from `phase` (include/dop.h:11-12);
 *   native bytes MSB first, a trailing partial byte left-aligned.
 * A decision is 1 when the float is >= 0.
 */
#include "oracle.h"

#include <string.h>

#define MARK_A 0x05u
#define MARK_B 0xFAu

int ora_dop_pack_i24(const float *bits, uint8_t *out, size_t n, int phase)
{
    if (!bits || !out || n == 0) return phase;
    size_t frames = n / 16;
    for (size_t f = 0; f < frames; f++) {
        unsigned w = 0;
        for (int b = 0; b < 16; b++)
            w = (w << 1) | (bits[16 * f + (size_t)b] >= 0.0f ? 1u : 0u);
        out[3 * f + 0] = (uint8_t)(w & 0xFFu);
        out[3 * f + 1] = (uint8_t)(w >> 8);
        out[3 * f + 2] = (uint8_t)(((f + (size_t)phase) & 1u) ? MARK_B : MARK_A);
    }
    return (int)((frames + (size_t)phase) & 1u);
}

void ora_bits_pack(const float *src, uint8_t *dst, size_t n)
{
    if (!src || !dst || n == 0) return;
    for (size_t i = 0; i < (n + 7) / 8; i++) {
        unsigned byte = 0;
        for (int b = 0; b < 8; b++) {
            size_t k = 8 * i + (size_t)b;
            if (k < n && src[k] >= 0.0f) byte |= 0x80u >> b;
        }
        dst[i] = (uint8_t)byte;
    }
}

/* Same packers over 0/1 decision bytes (the GPU's native decision format). */
int ora_dop_pack_u8(const uint8_t *bits, uint8_t *out, size_t n, int phase)
{
    if (!bits || !out || n == 0) return phase;
    size_t frames = n / 16;
    for (size_t f = 0; f < frames; f++) {
        unsigned w = 0;
        for (int b = 0; b < 16; b++) w = (w << 1) | (bits[16 * f + (size_t)b] & 1u);
        out[3 * f + 0] = (uint8_t)(w & 0xFFu);
        out[3 * f + 1] = (uint8_t)(w >> 8);
        out[3 * f + 2] = (uint8_t)(((f + (size_t)phase) & 1u) ? MARK_B : MARK_A);
    }
    return (int)((frames + (size_t)phase) & 1u);
}

void ora_bits_pack_u8(const uint8_t *bits, uint8_t *dst, size_t n)
{
    if (!bits || !dst || n == 0) return;
    for (size_t i = 0; i < (n + 7) / 8; i++) {
        unsigned byte = 0;
        for (int b = 0; b < 8; b++) {
            size_t k = 8 * i + (size_t)b;
            if (k < n && (bits[k] & 1u)) byte |= 0x80u >> b;
        }
        dst[i] = (uint8_t)byte;
    }
}

/* DSF payload (tools/dsd_encode.c:90-98 pack_dsd_lsb, :238-256 the 4096-byte
 * block padding; channels interleaved block by block per the DSF format):
 * [block][channel][4096], decision k of a byte at bit k.  Returns bytes. */
size_t ora_pack_dsf_u8(const uint8_t *bits, size_t stride, int nch, size_t n, uint8_t *out)
{
    size_t bytes = (n + 7) / 8, blocks = (bytes + 4095) / 4096;
    size_t total = blocks * 4096 * (size_t)nch;
    memset(out, 0, total);
    for (int c = 0; c < nch; c++)
        for (size_t i = 0; i < n; i++)
            if (bits[(size_t)c * stride + i] & 1u) {
                size_t byte = i / 8;
                out[(byte / 4096) * 4096 * (size_t)nch + (size_t)c * 4096 + byte % 4096] |=
                    (uint8_t)(1u << (i % 8));
            }
    return total;
}

/* DFF payload (tools/dsd_encode.c:80-88 pack_dsd_msb; channels interleaved
 * byte by byte per DSDIFF): [byte][channel], decision k of a byte at bit 7-k. */
size_t ora_pack_dff_u8(const uint8_t *bits, size_t stride, int nch, size_t n, uint8_t *out)
{
    size_t bytes = (n + 7) / 8, total = bytes * (size_t)nch;
    memset(out, 0, total);
    for (int c = 0; c < nch; c++)
        for (size_t i = 0; i < n; i++)
            if (bits[(size_t)c * stride + i] & 1u)
                out[(i / 8) * (size_t)nch + (size_t)c] |= (uint8_t)(0x80u >> (i % 8));
    return total;
}
