/* The code generator's interface (codegen.c): programs to CUDA C for NVRTC. */
#ifndef TC_CODEGEN_H
#define TC_CODEGEN_H

#include "tc_host.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The logic work of one 32-lane word in a generated enumeration kernel, as the code generator
   lays it out: LUTs run at every step, LUTs run once per stretch of stretch_steps steps, and the
   bit-sliced compare of the outputs (equiv: one XOR-OR per output; search: one op per output
   bit; a separable spec: its carry chain, 4 or 5 ops per bit above the step part's trailing
   zeros and 1 below; -1 when the spec is evaluated per lane, which is not counted).  With
   ticks > 1 or the mapping off, luts_per_step counts the NAND instructions instead. */
typedef struct {
    int luts_per_step, luts_per_stretch, stretch_steps, compare_ops;
} TcGenWork;

typedef struct {
    int             mode;       /* EN_VERIFY, EN_EQUIV, EN_SEARCH */
    const Program  *a, *b;      /* b: equiv */
    const uint32_t *b_inputs;   /* equiv: b's input cell for each of a's inputs, by name */
    const int      *out_map;    /* equiv: b's output index for each of a's outputs */
    const TcSpec   *spec;       /* verify, search */
    uint64_t        target;     /* search: the constant right side */
    unsigned        ticks;
    int             block;      /* threads per block */
    int             no_map;     /* 1: keep the NAND/STO body as written (no LOP3 mapping) */
    int             step_bits;  /* 3..5: the stretch length to use; 0: the cost model's choice */
    TcGenWork      *work;       /* out, when not NULL: the kernel's work per word */
} TcGenEnum;

/* The argument block of the generated kernel `tc_enum`, in one place: the host launchers declare
   TcEnumArgs from it with C's types, and tc_codegen_enum writes the same fields, as text, into the
   generated source with its own names for the types (u64, u32), so the two layouts cannot drift
   apart.  hits: one counter; list: 16 hits per warp; count: hits kept per warp. */
#define TC_ENUM_ARGS_FIELDS(u64, u32)                                                       \
    u64 words, space, per_warp;                                                             \
    u32 parts, part, nsel, pad;                                                             \
    u64 *hits;                                                                              \
    u64 *list;                                                                              \
    u32 *count;
#define TC_TEXT_(...) #__VA_ARGS__
#define TC_TEXT(...) TC_TEXT_(__VA_ARGS__)

typedef struct {
    TC_ENUM_ARGS_FIELDS(uint64_t, uint32_t)
} TcEnumArgs;

/* CUDA C for the enumeration kernel `tc_enum` (malloc'd; *len gets its length).  The per-word
   functions are plain C when TC_HOST_EMULATION is defined, so the tests can compile the same
   text for the host: tc_outer(cword, &inv) (what a stretch of steps shares), tc_inner(word, &inv)
   -> hit mask, tc_word(word) (the two for one word) and tc_unperm(y) (the assignment that
   enumeration index y stands for). */
char *tc_codegen_enum(const TcGenEnum *g, size_t *len);

/* Can the PTX writer (ptxgen.c) make this job's kernel?  Equivalence and search jobs of one tick,
   LUT-mapped. */
int   tc_ptx_enum_ok(const TcGenEnum *g);
/* PTX for the enumeration kernels of n such jobs (malloc'd; *len gets its length): one entry
   `tc_enum` for n = 1, else tc_enum_0 .. tc_enum_<n-1>, for `.target` target ("sm_103a"), each
   taking TcEnumArgs as the CUDA C kernel does.  work[k], when work is not NULL, gets kernel k's
   work per word. */
char *tc_ptx_enum(TcGenEnum *const *g, int n, const char *target, TcGenWork *work, size_t *len);

/* CUDA C for the truth-table kernel `tc_table` of a program without id or link cells. */
char *tc_codegen_table(const Program *p, unsigned ticks, int block, size_t *len);

/* CUDA C for the cube kernels of a program with id/link cells (cube.c). */
/* A program's closing copies as the cube plans them (cube.c): 1 with the copy segment's first
   instruction in *from and the second memory variant's cell map in slot1. */
int   tc_cube_copy_plan(const Program *p, size_t *from, uint32_t *slot1);
/* The source of every kernel of a cube's pass in memory variant 0 or 1, as the cube compiles them
   (NULL when the program has no variant 1); *nk gets the kernel count. */
char *tc_cube_source(const Program *p, unsigned variant, unsigned *nk, size_t *len);
char *tc_codegen_cube(const Program *p, const size_t *seg_first, unsigned nseg, int block,
                      size_t *len);

#ifdef __cplusplus
}
#endif
#endif
