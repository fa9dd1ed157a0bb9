/* tesseract_model.h — the host-side program model that ships with the GB300 engine: programs,
   the assembler, the gate builder and the workload generators, in plain C.

   These are the engine's own implementations of the reference's host helpers, with a tc_ prefix
   so that they link next to the reference's.  Each gives the same Program, cell for cell and
   instruction for instruction, as the reference function it names.  Programs returned here are
   freed with tc_program_free. */
#ifndef TESSERACT_MODEL_H
#define TESSERACT_MODEL_H

#include "tesseract_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/asm.c:767-801 and src/isa.h:48-62 */
void     tc_program_free(Program *p);
int      tc_program_find_cell(const Program *p, const char *name, uint32_t *addr);
int      tc_program_readonly(const Program *p, uint32_t cell);
uint32_t tc_program_resolve(const Program *p, uint32_t cell, unsigned *mask);
unsigned tc_program_dims(const Program *p);
int      tc_program_id_name(const char *name);
/* Writes the program as assembly text (src/build.c:432-444); returns bytes written, or the
   length needed when buf is too small (buf may be NULL with len 0). */
size_t   tc_program_print(const Program *p, char *buf, size_t len);
/* Deep copy (names included). */
int      tc_program_copy(const Program *src, Program *dst);

/* The assembler (src/asm.h:7-17): same language, same cell numbering, same @local names. */
int tc_asm_string(const char *src, const char *name, const char *base_dir, Program *out,
                  char *err, size_t errlen);
int tc_asm_file(const char *path, Program *out, char *err, size_t errlen);

/* Generators (src/gen.h, src/tester.h:18): the same instruction sequences as the reference's
   gen_mul, gen_hash, gen_life, gen_life_cube, random_program. */
void     tc_gen_mul(Program *p, int bits);
int      tc_gen_hash(Program *p, int bits, int rounds);
uint64_t tc_toyhash(uint64_t x, int bits, int rounds);
void     tc_gen_life(Program *p, int w, int h, uint32_t *board);
void     tc_gen_life_cube(Program *p, int w, int h, int rbits, int cbits, uint32_t *board);
/* The big-cube demos of `alpha cube --dims D` (src/cubedemo.c:398-548), for 2^dims machines:
   any (.in x, .out r: the OR of x over all machines), rank (.in x, .out p0.. t0..: how many
   machines below this one, and in all, have x = 1), sort (.in/.out v0..v7: bitonic sort, machine
   k ends with the k-th smallest byte). */
void     tc_gen_cube_any(Program *p, int dims);
void     tc_gen_cube_rank(Program *p, int dims);
void     tc_gen_cube_sort(Program *p, int dims);
/* max (.in v0..v7, .out m0..m7: the largest byte everywhere), anf (.in/.out f: the Möbius
   transform of a truth table, src/cubedemo.c:194-210), walsh (.in f, .out w0..: the
   Walsh-Hadamard spectrum, dims + 3 bits), ring (.in/.out x: one step of Rule 110 on the
   machines as a Gray-coded ring, src/cubedemo.c:286-306). */
void     tc_gen_cube_max(Program *p, int dims);
void     tc_gen_cube_anf(Program *p, int dims);
void     tc_gen_cube_walsh(Program *p, int dims);
void     tc_gen_cube_ring(Program *p, int dims);
/* pack (.in/.out v0..v7 h: the bytes of the machines with h = 1 gathered, in order, into the
   first machines, which end with h = 1, src/cubedemo.c:134-151), xorconv (.in f g, .out h0..:
   h(k) = how many j have f(j) = g(j ^ k) = 1, dims + 1 bits, by Walsh-Hadamard spectra,
   src/cubedemo.c:231-251). */
void     tc_gen_cube_pack(Program *p, int dims);
void     tc_gen_cube_xorconv(Program *p, int dims);
/* polymul (dims 9..11): .in a0.. b0.. zf<d>_0.. zi<d>_0.., .out c0..: c = a b in
   Z_12289[x]/(x^(2^dims) + 1), one coefficient per machine, by the number-theoretic transform
   (the reference's demo, src/gen.c:456-669, src/cubedemo.c:253-284); zf and zi are the forward
   and inverse twiddles of each round times 2^14 mod 12289, as cuda_cube_demo sets them. */
void     tc_gen_cube_polymul(Program *p, int dims);
unsigned tc_grid_machine(unsigned row, unsigned col, int cbits);
void     tc_random_program(Program *p, uint32_t cells, size_t len, uint64_t seed);
/* Random program with `width` input cells (.in w0.., never written) beside `cells` working cells
   (.out c0..): the input-width extension the batched equivalence workload needs; same
   splitmix64 stream as random_program. */
void     tc_random_program_in(Program *p, uint32_t cells, uint32_t width, size_t len,
                              uint64_t seed);
/* A copy of p rewritten by local NAND identities (double negation, commuted NAND pairs,
   De Morgan through a scratch cell) chosen by splitmix64(seed): the same function, a different
   program.  mutate != 0 also flips one instruction's operand, which normally changes it. */
void     tc_rewrite_program(const Program *p, Program *out, uint64_t seed, int mutate);

#ifdef __cplusplus
}
#endif
#endif
