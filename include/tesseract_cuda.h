/* tesseract_cuda.h — the C ABI of the GB300 engine for Tesseract's bit-sliced NAND/STO machine.

   This is `--engine cuda`: it sits beside the reference's ref, lanes and jit engines and takes the
   same program format, the same lane numbering and the same result structures.  Everything below
   is plain C: pointers, sizes and the reference's own structs.  No C++ or CUDA type crosses the
   boundary.  Every entry point returns 1 on success, or 0 with a message in `err` (the reference's
   convention, src/enum.c:248-260, src/jit.c:672-674).

   The data types are byte-for-byte the reference's, so a Program, Enum, EnumResult or
   CheckResult built by the reference's own code can be passed straight in:
     Instr, CellInfo, Program   src/isa.h:14-46
     Enum, EnumResult           src/enum.h:15-36
     CheckResult                src/check.h:8-20
     Spec (opaque here)         layout of src/spec.c:20-29
   When the reference's headers are included first, their definitions are used and the ones here
   are skipped (same include guards). */
#ifndef TESSERACT_CUDA_H
#define TESSERACT_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- the program model (src/isa.h:8-46) -------------------------------------------------- */
#ifndef ALPHA_ISA_H
#define ALPHA_ISA_H
enum { OP_NAND = 0, OP_STO = 1 };
enum { CELL_ZERO = 0, CELL_ONE = 1, CELL_FIRST_FREE = 2 };
typedef struct {
    uint8_t  op;    /* OP_NAND or OP_STO */
    uint32_t addr;  /* cell address */
} Instr;
enum { CUBE_DIMS = 9, CUBE_SIZE = 1 << CUBE_DIMS, CUBE_MAX_DIMS = 16,
       CUBE_MAX_GROUPS = 1 << (CUBE_MAX_DIMS - CUBE_DIMS) };
enum { CK_PLAIN, CK_ID, CK_LINK };
typedef struct {
    uint8_t  kind;  /* CK_PLAIN, CK_ID (bit `dim` of the machine number), CK_LINK */
    uint8_t  dim;
    uint32_t src;   /* CK_LINK: the cell read in machine k XOR 2^dim */
} CellInfo;
typedef struct {
    Instr    *code;
    size_t    len;
    uint32_t  ncells;      /* cells used, including ZERO and ONE */
    char    **cell_names;
    uint32_t *inputs;      /* .in cells, in declaration order */
    size_t    ninputs;
    uint32_t *outputs;     /* .out cells, in declaration order */
    size_t    noutputs;
    CellInfo *special;     /* NULL when the program has no id or link cells */
} Program;
#endif

/* ---- specifications (src/spec.h) ---------------------------------------------------------- */
#ifndef ALPHA_SPEC_H
#define ALPHA_SPEC_H
typedef struct Spec Spec;
#endif

/* ---- exhaustive enumeration (src/enum.h:10-36) ------------------------------------------- */
#ifndef ALPHA_ENUM_H
#define ALPHA_ENUM_H
enum { EN_VERIFY, EN_EQUIV, EN_SEARCH };
#define EN_SHOW    16  /* hits kept: the smallest assignments */
#define EN_MAX_IN  46  /* inputs */
typedef struct {
    int                  mode;
    const Program       *a, *b;   /* b: equiv only; inputs and outputs matched by name */
    const Spec          *spec;    /* verify: outputs = expression; search: outputs = constant */
    unsigned             ticks;   /* passes per assignment */
    int                  threads; /* CPU engines only; ignored on the GPU */
    int                  idle;    /* CPU engines only; ignored on the GPU */
    const unsigned char *excluded;
    int                  part, part_end, parts;  /* shares part..part_end of `parts` */
} Enum;
typedef struct {
    uint64_t space;  /* assignments in total: 2^inputs */
    uint64_t tried;  /* assignments run (this share) */
    uint64_t hits;   /* verify, equiv: mismatches; search: matches */
    uint64_t hit[EN_SHOW];
    int      nhit;
    double   seconds;
    uint64_t ops;    /* 1-bit operations: ticks x length x 512 per pass, as the reference counts */
    int      threads;
} EnumResult;
#endif

/* ---- engine-vs-reference check (src/check.h:8-20) ---------------------------------------- */
#ifndef ALPHA_CHECK_H
#define ALPHA_CHECK_H
typedef struct {
    int      ok;
    uint64_t compared;  /* lane states compared */
    uint64_t tick;      /* 1-based tick of the first difference */
    long     pc;        /* -1: end of the tick */
    unsigned lane;      /* machine number */
    long     cell;      /* cell address, or -1 = RR */
    unsigned want;      /* reference machine */
    unsigned got;       /* this engine */
} CheckResult;
#endif

/* ---- the superoptimizer (src/super.h:19-72) ---------------------------------------------- */
#ifndef ALPHA_SUPER_H
#define ALPHA_SUPER_H
enum { SUPER_VARS = 6, SUPER_CELLS = 16, SUPER_LEN = 64, SUPER_NAME = 24 };
typedef struct {
    int      nvars;      /* input variables; truth tables have 2^nvars rows */
    uint64_t mask;       /* the 2^nvars rows */
    int      rr_in;      /* RR's first value is variable 0 */
    int      rr_out;     /* RR must end as rr_target */
    uint64_t rr_target;
    int      ncells;
    struct {
        char     name[SUPER_NAME];
        int      in, out;   /* holds init at the start / must hold target at the end */
        uint64_t init, target;
        uint32_t alias;     /* bit i: this output may share input cell i's cell */
        int      sym_prev;  /* interchangeable inputs: read only after cell sym_prev; -1 none */
    } cell[SUPER_CELLS];
} SuperSpec;
typedef struct {
    int len;
    struct {
        uint8_t op;  /* OP_NAND or OP_STO */
        char    cell[SUPER_NAME];
    } code[SUPER_LEN];
} SuperProg;
typedef struct {
    int threads;      /* CPU search only; ignored on the GPU */
    int part, parts;  /* CPU cluster shares; the GPU search runs the whole tree */
    int max_cost;
    int quiet;
} SuperOpts;
typedef struct {
    int       found, cost;    /* the shortest program, and its length */
    int       below;          /* every program shorter than this was tried: none exists */
    int       contradiction;  /* found one shorter than `below`: the search is wrong */
    SuperProg prog;
    uint64_t  nodes;
    double    seconds;
} SuperResult;
#endif

/* ========================================================================================== */
/* Entry points.  Each names the reference interface it replaces.                             */
/* ========================================================================================== */

/* Library and device.  cuda_device_info writes "NVIDIA GB300, 152 SMs, sm_103" style text. */
int  cuda_engine_init(int device, char *err, size_t errlen);
int  cuda_device_info(char *buf, size_t len);

/* Measurement.  cuda_last_launch reports the last kernel launch of this process: device time
   (CUDA events on the engine's stream), registers per thread, local-memory bytes per thread
   (spills), grid and block, and the NVRTC compile time of its module (cached = 1 when the module
   came from the cache).  cuda_lop3_peak measures the device's 3-input logic issue rate with a
   microbenchmark: 32-bit LOP3 operations per second (each is 32 one-bit lane operations).
   For a generated enumeration kernel the launch stats also give its logic work per 32-lane word
   as the code generator laid it out: LUTs run every step, LUTs run once per stretch of
   stretch_steps steps, and the bit-sliced output compare (compare_ops, -1 when the spec is
   evaluated per lane); logic_ops_per_word = luts_per_step + luts_per_stretch / stretch_steps +
   compare_ops, or 0 when not counted.  ptx = 1 when the kernel was built from PTX that the engine
   writes directly (the quick-start build of an equivalence or search job), 0 for CUDA C.
   Neither has a counterpart in the reference, whose engines run on the CPU. */
typedef struct {
    double   kernel_ms;
    int      regs, local_bytes;
    unsigned grid, block;
    double   compile_seconds;
    int      cached;
    int      luts_per_step, luts_per_stretch, stretch_steps, compare_ops;
    double   logic_ops_per_word;
    int      ptx;
} CudaLaunchStats;
int  cuda_last_launch(CudaLaunchStats *s);
int  cuda_lop3_peak(double *ops_per_second, double *seconds, char *err, size_t errlen);

/* Specifications.  Replaces spec_parse / spec_free / spec_width / spec_out_cell / spec_value
   (src/spec.h:22-29) with the same grammar, errors and results; the Spec it returns has the
   layout of src/spec.c:20-29, so a Spec from the reference's spec_parse is accepted as well. */
Spec    *cuda_spec_parse(const char *text, const Program *p, int inputs_allowed, char *err,
                         size_t errlen);
void     cuda_spec_free(Spec *s);
int      cuda_spec_width(const Spec *s);
uint32_t cuda_spec_out_cell(const Spec *s, int bit);
uint64_t cuda_spec_value(const Spec *s, uint64_t x);

/* Compiled code.  Replaces jit_compile / jit_free (src/jit.h:45-48): the program becomes one
   CUDA kernel per pass, generated as CUDA C and compiled by NVRTC for sm_103a; compiled modules
   are cached by content hash for the life of the process. */
typedef struct CudaCode CudaCode;
int  cuda_compile(const Program *p, CudaCode **out, char *err, size_t errlen);
void cuda_free(CudaCode *c);

/* verify / equiv / search over every assignment.  Replaces enum_run (src/enum.h:37,
   src/enum.c:244-332): same refusals, same --part shares, same hits, same 16 smallest hits,
   same ops accounting.  r->threads reports the GPU threads used; r->seconds the wall time of
   the device work. */
int  cuda_enum_run(const Enum *e, EnumResult *r, char *err, size_t errlen);
void cuda_enum_add_hit(EnumResult *r, uint64_t x);   /* enum_add_hit, src/enum.c:31-46 */

/* The autotuner: kernels of job e for 128, 256 and 512 threads per block and, where the work
   splits into stretches, stretches of 8, 16 and 32 steps (step_bits 3..5; 0: not split) are
   compiled in parallel, checked to give the same result and timed on the job (or on the share of
   its chunks that takes about 20 ms: probe_fraction); the fastest is kept as the job's kernel
   for every later launch of it in this process (cuda_enum_run, batches, serving,
   cuda_enum_run_static).  cand[i].ms is candidate i's best of three, -1 when it did not compile.
   No counterpart in the reference. */
typedef struct {
    int    n, ncand, best;
    struct {
        int    block, step_bits;
        double ms;
    } cand[9];
    double probe_fraction;
} CudaTune;
int  cuda_enum_tune(const Enum *e, CudaTune *t, char *err, size_t errlen);
/* Adds the result of one share (--part) into a total, as merge_raw does (src/work.c:341-371):
   the host side of running shares on several GPUs or machines.  Needs no GPU. */
void cuda_enum_merge(EnumResult *into, const EnumResult *part);

/* cuda_enum_run without allocation: the same job, kernel and results, with the workspace (hit
   counter, per-warp hit lists and counts) in a fixed 2.1 MB device array for at most 16,384
   warps instead of buffers grown by cudaMalloc.  For callers that cannot allocate: a serving loop
   whose device memory is handed out to admitted jobs, or one with kernels in flight on other
   streams that a cudaFree would wait for.  It compiles nothing: the job's kernel must have been
   loaded by an earlier cuda_enum_run of the same job, else it fails with an error; so does a
   launch needing more warps than the array holds.  The first call on a device looks up the
   array's address (make it before any stream capture).  Calls share the array: calls that
   overlap on the GPU race.  No counterpart in the reference. */
int  cuda_enum_run_static(const Enum *e, EnumResult *r, char *err, size_t errlen);

/* Batches.  Runs every job of an array of enumerations (verify, equiv, search; whole spaces, no
   --part) in one persistent launch of a precompiled interpreter kernel fed from a device work
   queue, and writes one EnumResult per job with the same fields as cuda_enum_run.  No per-program
   compilation, so thousands of different programs cost one launch; jobs are refused when their
   cells exceed the interpreter's 255 shared-memory slots.  No counterpart in the reference, which
   runs one enumeration per command. */
int  cuda_batch_run(const Enum *const *jobs, int njobs, EnumResult *results, char *err,
                    size_t errlen);
/* The last cuda_batch_run: jobs, how many ran as generated kernels and how many on the
   interpreter, the compile threads it used, how many jobs its plan sent to generated code and how
   many of those the interpreter took back (still waiting for a compile thread when it ran out of
   work), its wall time, in seconds from its start when the interpreter's first launch went out
   (after packing) and when the last interpreted and the last compiled job finished, the compile
   threads' busy seconds summed (code generation and NVRTC), the seconds the host loop spent
   loading the compiled modules (a load waits for the device's running work), and when the host
   loop had every result. */
typedef struct {
    int    jobs, compiled, interpreted, compile_threads, planned, taken_back;
    double seconds, interpreter_start, interpreter_end, compiled_end, compile_busy, compile_load,
        loop_end;
} CudaBatchStats;
int  cuda_batch_stats(CudaBatchStats *s);
/* Compiles and loads, on the host's cores less two, the kernel of every job of an array that a
   batch could run as generated code (whole spaces whose work pays for a launch; optimised, as a
   served job's: PTX through ptxas -O3 for equivalence and search, NVRTC -O2 for the rest), so
   that a later cuda_batch_run of the same jobs finds every such kernel cached; *prepared (when
   not NULL) gets how many.  For job sets that run repeatedly. */
int  cuda_batch_prepare(const Enum *const *jobs, int njobs, int *prepared, char *err,
                        size_t errlen);

/* The superoptimizer.  cuda_super_parse replaces super_parse (src/super.c:225-371): same
   language, same SuperSpec.  cuda_super_search replaces super_search (src/super.c:821-896):
   iterative deepening over the budget from the same lower bound, the same chain-program model
   and pruning rules, every budget below the answer searched in full on the GPU, so `cost` and
   `below` mean what they mean there.  Node counts differ: the search visits only children
   within the bound, and its transposition table is one table shared by every warp.
   cuda_super_check replaces super_check (src/super.c:908-1001). */
int  cuda_super_parse(const char *text, SuperSpec *sp, char *err, size_t errlen);
int  cuda_super_search(const SuperSpec *sp, const SuperOpts *o, SuperResult *r, char *err,
                       size_t errlen);
int  cuda_super_check(const SuperSpec *sp, const SuperProg *p, char *err, size_t errlen);

/* Serving.  Jobs arrive at arrival[i] seconds after the call starts (sorted) and each runs on
   one of two engines, chosen when it arrives (`route`; automatic by default: the generated-kernel
   engine when the GPU time it saves over the interpreter outweighs the job's compile time spread
   over the compile threads):
   - the batched interpreter: jobs are admitted while fewer than max_inflight_jobs are on the
     device and their packed footprint fits max_device_bytes, and run in waves of up to
     max_wave_jobs, each one persistent launch on one of `streams` streams taking `share` of the
     GPU's resident blocks, so waves overlap on the device;
   - the generated-kernel engine of cuda_enum_run: compile_threads host threads generate and
     compile (cached by what the generator reads) while earlier jobs run; up to compiled_slots
     compiled jobs are on the device at once, each on its own stream and preallocated workspace.
   start[i] / finish[i] get the seconds (from the call's start) when job i was launched and when
   its result was known on the host; results[i] its result, the same as cuda_enum_run's;
   engine_used[i] (may be NULL) 0 for the interpreter, 1 for generated code.  Zero fields take
   defaults (4 streams, 4096 jobs, 8 GiB, 1024 jobs, 0.5, 12 threads, 4 slots, automatic
   routing).  No counterpart in the reference. */
#define CUDA_SERVE_AUTO        0
#define CUDA_SERVE_INTERPRETER 1
#define CUDA_SERVE_COMPILED    2
typedef struct {
    int    streams;
    int    max_inflight_jobs;
    size_t max_device_bytes;
    int    max_wave_jobs;
    double share;
    int    compile_threads;
    int    compiled_slots;
    int    route;
} CudaServeOpts;
int  cuda_serve_run(const Enum *const *jobs, const double *arrival, int njobs,
                    const CudaServeOpts *opts, double *start, double *finish,
                    EnumResult *results, int *engine_used, char *err, size_t errlen);

/* Truth tables.  Replaces table_lanes (src/main.c:297-322) for `run --table --engine cuda`:
   every row of a program without id or link cells (1 to 20 .in cells; the first .in cell is the
   row's high bit) from the reset state, `ticks` passes, then the .out cells, or RR when there are
   none (src/main.c:219-258).  vals gets 2^ninputs rows of max(noutputs, 1) bytes, each 0 or 1. */
int  cuda_table(const Program *p, unsigned ticks, uint8_t *vals, char *err, size_t errlen);

/* Tester 1: what do random 1-bit computers do?  The reference's configuration and result
   (src/tester.h:7-51, same layout, its include guard), and cuda_t1_run in place of t1_run
   (src/tester.h:55, src/tester.c:235-275): every random program of every size runs from 512
   random states on the GPU and Brent's algorithm finds the cycle each run ends in.  Returns the
   wall seconds (-1 with a message in err); *threads gets 1.  With cfg->programs > 0 the
   histograms, pass counts and longest cycles equal a one-thread reference run's. */
#ifndef ALPHA_TESTER_H
#define ALPHA_TESTER_H
#define T1_BUCKETS 64  /* bucket b: cycle length in (2^(b-1), 2^b]; the last one: not found */
#define T1_SIZES   32
typedef struct {
    uint32_t cells;
    size_t   len;
    uint64_t programs, starts, passes;
    uint64_t unfinished;
    uint64_t hist[T1_BUCKETS];
    uint64_t longest, longest_seed;
} T1Size;
typedef struct {
    uint32_t             cells[T1_SIZES];
    int                  nsizes;
    double               ratio;
    uint64_t             programs;
    double               seconds;
    uint64_t             max_passes;
    uint64_t             seed;
    int                  threads;
    int                  idle;
    const unsigned char *excluded;
} T1Config;
#endif
double cuda_t1_run(const T1Config *cfg, T1Size *out, int *threads, char *err, size_t errlen);

/* Random-state parity against the reference semantics.  Replaces
   check_lanes(p, jit, seed, ticks, 0, r) (src/check.h:25, src/check.c:52-113): every machine of
   the program's cube gets the same random state from splitmix64(seed) as there, runs `ticks`
   passes on the GPU, and the full state (RR and every cell) is compared after each tick with the
   reference machine, run on the host. */
int  cuda_check(const Program *p, uint64_t seed, unsigned ticks, CheckResult *r, char *err,
                size_t errlen);

/* The cube (programs with id and link cells, up to 2^16 machines).  Replaces LaneCube +
   jit_cube_run (src/lanes.h:66-80, src/jit.h:58-61).  The state lives on the device.  Lines use
   the reference's layout: per group of 512 machines, `ncells` lines of 8 uint64 each, machine k
   of the group at bit k%64 of word k/64 (src/lanes.h:13-15), and one line for RR. */
typedef struct CudaCube CudaCube;
int  cuda_cube_new(const Program *p, CudaCube **out, char *err, size_t errlen);
void cuda_cube_free(CudaCube *c);
unsigned cuda_cube_groups(const CudaCube *c);
/* cuda_cube_segments: the segments the ISA's rule cuts a pass into (a cut wherever a cell written
   in the segment is read across dimension 9 or up, docs/ISA.md step 7f), as the reference's
   engines cut it; this engine itself cuts only from dimension 10 up (1,024 machines run in
   lockstep inside one warp) and cuda_cube_kernels counts its launches per pass. */
unsigned cuda_cube_segments(const CudaCube *c);
int  cuda_cube_load(CudaCube *c, unsigned group, const uint64_t *mem_lines, const uint64_t *rr_line,
                    char *err, size_t errlen);
int  cuda_cube_store(const CudaCube *c, unsigned group, uint64_t *mem_lines, uint64_t *rr_line,
                     char *err, size_t errlen);
int  cuda_cube_run(CudaCube *c, uint64_t passes, char *err, size_t errlen);
/* The cube's autotuner: the kernels whose blocks each run one warp group's code are compiled for
   4 and 8 warps per block and 1, 2 and 4 runs of words per block (as the cube's size allows; the
   present shape first), each variant is run for probe_passes passes from the cube's present
   state (saved before, restored after: the state is unchanged), and the fastest is kept for every
   later pass.  cand[i].ms is variant i's time.  No counterpart in the reference. */
#define CUBE_TUNE_MAX 8
typedef struct {
    int      n, best;
    struct {
        unsigned warps, iters;
        double   ms;
    } cand[CUBE_TUNE_MAX];
    unsigned probe_passes;
} CudaCubeTune;
int  cuda_cube_tune(CudaCube *c, unsigned probe_passes, CudaCubeTune *t, char *err,
                    size_t errlen);
/* The whole cube at once, cell-major: cell c of machine m is bit m % 32 of word c * W + m / 32,
   W = machines / 32 (ncells x W words), and RR as W words; ZERO and ONE keep their values.
   cuda_cube_kernels: kernel launches per pass (segments, long ones split).
   cuda_cube_closing_copies: how many of them are the pass's closing copies (A <- B: a Life
   board taking its next generation), which a run leaves out of every pass but its last by
   exchanging A's and B's memory in alternate passes (0: the program has none, or they do not
   qualify). */
int  cuda_cube_read_words(const CudaCube *c, uint32_t *mem, uint32_t *rr, char *err,
                          size_t errlen);
int  cuda_cube_write_words(CudaCube *c, const uint32_t *mem, const uint32_t *rr, char *err,
                           size_t errlen);
unsigned cuda_cube_kernels(const CudaCube *c);
unsigned cuda_cube_closing_copies(const CudaCube *c);

/* `alpha cube DEMO --dims D` (src/cubedemo.c:549-623) on the GPU cube: builds demo any, rank,
   sort or life for 2^dims machines (dims 9..16), runs `checks` rounds of random inputs one pass
   each and checks every machine against plain C (a sorted array, prefix counts, plain Life),
   then times passes for about `seconds`.  r->ok is 0 when a check failed. */
typedef struct {
    char     what[96];
    size_t   instr;
    unsigned segs, kernels;
    int      ok;
    double   pass_seconds, passes_per_second;
} CudaDemoResult;
int  cuda_cube_demo(const char *name, int dims, int checks, double seconds, CudaDemoResult *r,
                    char *err, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif
