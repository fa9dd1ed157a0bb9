/* Helpers of the command-line tool that live in the library (cli_support.c). */
#ifndef TC_CLI_SUPPORT_H
#define TC_CLI_SUPPORT_H

#include <stddef.h>
#include <stdint.h>

#include "../../include/tesseract_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* `life`: 512 independent boards (cube = 0: gen_life, one lane each) or one board over a cube of
   2^dims machines in 2^rbits rows (cube = 1: gen_life_cube); size x size cells a board or tile. */
typedef struct {
    int                cube, dims, rbits, size;
    unsigned long long gens;
    uint64_t           seed;
} TcLifeRun;

typedef struct {
    size_t   len;                /* NAND/STO instructions per generation */
    unsigned segments, machines; /* the pass's segments on the cube engine; machines run */
    int      board_w, board_h;   /* the whole board (cube), or one board */
    double   gpu_ms;
    int      bad;                /* -1: equal to plain C Life; else the first board (512 boards)
                                    or row (cube) that differs */
    uint8_t *shown;              /* 512 boards: board 0 (size x size) as the engine left it;
                                    cube: the plain C board's top left rows x cols; free() it */
    int      rows, cols, alive;  /* cube: the corner's size; 512 boards: cells alive on board 0 */
} TcLifeResult;

int tc_life_run(const TcLifeRun *a, TcLifeResult *r, char *err, size_t errlen);

#ifdef __cplusplus
}
#endif
#endif
