/* Tester 1's packed format, shared by the host (tester.c) and the kernel (tester_kernels.cu). */
#ifndef TC_TESTER_H
#define TC_TESTER_H

#include <stdint.h>

/* One launch: programs k0 .. k0 + n - 1 of one machine size.  Each block makes its program
   itself (the reference's random_program from t1_program_seed) and adds its 512 runs to the
   size's histogram; per program it leaves the passes run and its longest cycle. */
typedef struct {
    uint64_t  seed;        /* the run's --seed */
    uint64_t  k0;          /* the first program's number */
    uint64_t  max_passes;
    uint32_t  cells;       /* writable cells; the machine has cells + 2 */
    uint32_t  len;         /* instructions per program */
    uint32_t  nsample;     /* sample cells compared first (up to 64) */
    uint32_t  pad;
    uint64_t *hist;        /* T1 buckets, added to with atomics */
    uint64_t *passes;      /* per program */
    uint64_t *longest;     /* per program: its longest cycle */
} TcT1Dev;

#endif
