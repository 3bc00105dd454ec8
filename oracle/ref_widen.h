/*
 * Test infrastructure only (oracle).  Force-included (gcc -include) when
 * oracle/Makefile compiles the reference's src/trellis.c for the widened
 * oracle: after the system headers are in, every uint32_t in the reference's
 * trellis types (sdm_state_t.path, sdm_context_t.trellis_mask) becomes a
 * 64-bit type, so a dedup mask of 48 or 64 bits can be represented.  Nothing
 * else about the reference code changes.
 */
#ifndef REF_WIDEN_H
#define REF_WIDEN_H
#include <stdint.h>
#include <stddef.h>
#include <stdbool.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <math.h>
#define uint32_t uint64_t
#endif
