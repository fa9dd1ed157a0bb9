/* Host-side program model of the GB300 engine: programs, the assembler, specifications, the gate
   builder and the workload generators.  Everything here is plain C11 and runs on the host; the
   device side lives in engine.cu.  Names carry a tc_ prefix so the library can be linked into the
   reference's own binary next to its program_* / spec_* / b_* functions. */
#ifndef TC_HOST_H
#define TC_HOST_H

#include <stdio.h>

#include "../../include/tesseract_cuda.h"
#include "../../include/tesseract_model.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The layout of a parsed specification: identical to the reference's private struct
   (src/spec.c:11-29), so that a Spec built there can be read here. */
enum { TS_NUM, TS_VAR, TS_ADD, TS_SUB, TS_MUL, TS_AND, TS_OR, TS_XOR, TS_SHL, TS_SHR, TS_NOT,
       TS_NEG };
#define TS_MAX_VARS  32
#define TS_MAX_RPN   256
#define TS_MAX_STACK 64
typedef struct {
    int      op;
    uint64_t v;
} TcSpecItem;
typedef struct {
    int        width;
    uint32_t   out[64];
    int        nvars;
    char       var_name[TS_MAX_VARS][64];
    int        var_bits[TS_MAX_VARS];
    int        var_pos[TS_MAX_VARS][64];  /* bit of x for each bit of the vector */
    TcSpecItem rpn[TS_MAX_RPN];
    int        nrpn, depth, max_depth;
} TcSpec;

void *tc_xmalloc(size_t n);
void *tc_xcalloc(size_t n, size_t k);
void *tc_xrealloc(void *p, size_t n);
char *tc_xstrdup(const char *s);
int   tc_same_name(const char *a, const char *b);  /* case-insensitive equality */
uint64_t tc_splitmix64(uint64_t *s);

/* Program text as the reference's program_print writes it (src/build.c:417-444). */
char *tc_program_text(const Program *p, size_t *len);

#ifdef __cplusplus
}
#endif
#endif
