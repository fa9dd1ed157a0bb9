/* Tester 1's packed format, shared by the host (tester.c) and the kernel (tester_kernels.cu). */
#ifndef TC_TESTER_H
#define TC_TESTER_H

#include <stdint.h>

typedef struct {
    uint64_t seed;     /* the program's seed: its instructions and its 512 starting states */
    uint32_t ncells;   /* cells + 2 (ZERO, ONE) */
    uint32_t len;      /* instructions */
    uint32_t code;     /* first instruction in the code array: (addr << 1) | op each */
    uint32_t sample;   /* first entry of its sample cells in the sample array */
    uint32_t nsample;
    uint32_t pad;
} TcT1Job;

typedef struct {
    const TcT1Job  *jobs;
    const uint32_t *code;
    const uint32_t *sample;
    uint64_t       *lam;     /* 512 per program: the cycle length each lane reached, or 0 */
    uint64_t       *passes;  /* per program: passes run */
    uint64_t        max_passes;
} TcT1Dev;

#endif
