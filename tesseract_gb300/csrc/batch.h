/* The batched engine's packed format, shared by the host packer (batch.c) and the persistent
   interpreter kernel (batch_kernels.cu).

   A job is one enumeration (verify, equiv or search) of one program or pair.  Its programs are
   packed into bundles of 64 bits, each a run of up to 4 NANDs followed by up to 3 STOs:
     byte 0        number of NANDs (low nibble) and of STOs (high nibble)
     bytes 1..4    NAND operands (slot numbers)
     bytes 5..7    STO targets
   Slots are the job's cells in shared memory, one 32-bit word per thread each: program a's cells
   first, then program b's; ZERO and ONE of each program are slots holding 0 and ~0.  A STO to a
   read-only cell is dropped while packing. */
#ifndef TC_BATCH_H
#define TC_BATCH_H

#include <stdint.h>

#define TC_BATCH_BLOCK 128         /* threads per block; one 32-lane word per thread */
#define TC_BATCH_UNIT_WORDS 4096   /* words per work unit: 131,072 assignments */
#define TC_BATCH_UNIT_WORDS_MIN 256 /* the smallest unit a small wave is cut into */
#define TC_BATCH_MAX_SLOTS 255
#define TC_BATCH_SHOW 16

typedef struct {
    uint64_t words;          /* 32-lane words in the job's space */
    uint64_t space;          /* assignments: 2^inputs */
    uint32_t code_a, nb_a;   /* first bundle and bundle count of program a */
    uint32_t code_b, nb_b;   /* program b (equiv), else 0 */
    uint32_t lists;          /* first entry in the list array: inputs, zero slots, compares */
    uint16_t n_in;           /* inputs: pairs (slot a, slot b) follow in the list array */
    uint16_t n_zero;         /* slots to clear before every word */
    uint16_t n_cmp;          /* equiv: pairs (slot a, slot b); search: (slot, target bit);
                                verify: output slots, lowest bit first */
    uint16_t slots;          /* slots in use */
    uint16_t one_a, one_b;   /* the ONE slots */
    uint8_t  mode;           /* EN_VERIFY, EN_EQUIV, EN_SEARCH */
    uint8_t  ticks;
    uint8_t  lut;            /* 1: code_a/nb_a are LOP3 ops (four words each, see below) */
    uint8_t  pad;
    uint32_t rpn;            /* verify: first item in the RPN array */
    uint16_t nrpn, nvars;
    uint32_t vars;           /* verify: first entry (per var: bits, then positions) */
    uint32_t first_unit;     /* its first work unit */
    uint32_t units;
    uint32_t unit_words;     /* words per work unit (the last may have fewer) */
    uint32_t pad2;
} TcBatchJob;

typedef struct {
    uint32_t op;             /* TS_* */
    uint32_t pad;
    uint64_t v;
} TcBatchRpn;

/* A LUT job (lut = 1, one tick) is the pass mapped onto 3-input LUTs (lutmap.c): op i is four
   words: the byte offsets in shared memory of its three operands, then the destination's byte
   offset with the truth table in the top 8 bits.  Its slots are values, not cells: slot 0 holds
   0, slot 1 ~0, slots 2.. the inputs, the others LUT results, reused once dead. */

/* The device arrays of one batch, passed to the kernel by value. */
struct TcBatchDev {
    const TcBatchJob   *jobs;
    const uint64_t     *code;
    const uint32_t     *luts;
    const uint16_t     *lists;
    const TcBatchRpn   *rpn;
    const uint8_t      *vars;
    const uint32_t     *unit_job;
    uint32_t            unit_base;   /* this launch takes units unit_base .. nunits - 1 */
    uint32_t            nunits;
    uint32_t           *next_unit;
    unsigned long long *hits;        /* per job */
    unsigned long long *unit_hits;   /* per unit, TC_BATCH_SHOW each */
    uint32_t           *unit_count;  /* per unit */
    uint32_t           *remaining;   /* per job: units not finished yet */
    unsigned long long *hits_out;    /* per job, host-mapped: the final count */
    uint32_t           *done;        /* per job, host-mapped: 1 once every unit is finished */
};

#endif
