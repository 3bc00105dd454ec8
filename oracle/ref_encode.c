/*
 * ORACLE — test infrastructure only (see oracle.h).
 *
 * Compiles the reference's offline encoder, tools/dsd_encode.c, where it lies
 * (the Makefile passes its path as REF_ENCODE_C) so that its file writers and
 * input reader can be called on known data:
 *   write_dsf / write_dff (tools/dsd_encode.c:164-292) with their packers
 *   pack_dsd_lsb / pack_dsd_msb (:80-98), and read_input (:118-162, which
 *   reads a WAV with src/wav_io.c and mixes it to mono).
 * The tool is Windows code: the three CRT names it uses are mapped to their
 * POSIX equivalents below.  Its FIR chain (src/fir.c) needs Intel IPP and is
 * not built; the stand-ins below only satisfy the linker (the encoder's main
 * is never called).
 */
#include <stdio.h>
#include <stdlib.h>
#include <strings.h>

#define fopen_s(pf, path, mode) ((*(pf) = fopen((path), (mode))) == NULL)
#define _stricmp strcasecmp
#define _atoi64 atoll

#include REF_ENCODE_C

int fir_chain_init(fir_chain_t *chain, uint32_t fs_in, uint32_t fs_out)
{
    (void)chain; (void)fs_in; (void)fs_out;
    return -1;
}

size_t fir_chain_process(fir_chain_t *chain, const float *in, float *out, size_t in_count)
{
    (void)chain; (void)in; (void)out; (void)in_count;
    return 0;
}

void fir_chain_free(fir_chain_t *chain) { (void)chain; }

int ref_write_dsf(const char *path, const float *dsd, size_t count, uint32_t rate)
{
    return write_dsf(path, dsd, count, rate);
}

int ref_write_dff(const char *path, const float *dsd, size_t count, uint32_t rate)
{
    return write_dff(path, dsd, count, rate);
}

/* read_input into a caller buffer: returns the sample count, or -1. */
long long ref_read_input(const char *path, float *out, size_t cap, uint32_t *rate)
{
    size_t n = 0;
    *rate = 0;
    float *buf = read_input(path, rate, &n);
    if (!buf) return -1;
    size_t k = n < cap ? n : cap;
    memcpy(out, buf, k * sizeof(float));
    free(buf);
    return (long long)n;
}

/* wav_read (src/wav_io.c:43-152): interleaved floats; returns frames or -1. */
long long ref_wav_read(const char *path, float *out, size_t cap, uint32_t *rate, int *channels)
{
    wav_data_t w;
    if (wav_read(path, &w) != 0) return -1;
    size_t total = (size_t)w.num_frames * w.channels;
    memcpy(out, w.samples, (total < cap ? total : cap) * sizeof(float));
    *rate = w.sample_rate;
    *channels = w.channels;
    long long frames = (long long)w.num_frames;
    wav_free(&w);
    return frames;
}

int ref_wav_write(const char *path, const float *samples, uint32_t frames, int channels, uint32_t rate)
{
    return wav_write(path, samples, frames, (uint16_t)channels, rate);
}
