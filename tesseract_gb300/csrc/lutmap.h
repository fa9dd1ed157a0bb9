/* NAND networks mapped onto 3-input LUTs (lutmap.c). */
#ifndef TC_LUTMAP_H
#define TC_LUTMAP_H

#include "tc_host.h"

#ifdef __cplusplus
extern "C" {
#endif

enum { TN_CONST, TN_LEAF, TN_NAND, TN_NOT };

typedef struct {
    int kind;
    int a, b;  /* fanins (NAND: a < b; NOT: a) ; CONST: a = value */
    int id;    /* LEAF: the caller's number for it */
} TcNode;

typedef struct TcNet TcNet;

TcNet *tc_net_new(void);        /* nodes 0 and 1 are the constants 0 and ~0 */
void   tc_net_free(TcNet *t);
int    tc_net_const(TcNet *t, int v);
int    tc_net_leaf(TcNet *t, int id);
int    tc_net_nand(TcNet *t, int a, int b);
int    tc_net_not(TcNet *t, int a);
int    tc_net_size(const TcNet *t);
const TcNode *tc_net_node(const TcNet *t, int i);

/* Maps the network onto 3-input LUTs covering `outputs`; order gets the chosen nodes in
   topological order (norder of them).  Returns the LUT count. */
int  tc_net_map(TcNet *t, const int *outputs, int nout, int *order, int *norder);
/* The LUT chosen for a mapped node: its leaves (node numbers, 1..3) and truth table over the
   lop3.b32 patterns 0xf0, 0xcc, 0xaa of leaves 0, 1, 2. */
void tc_net_lut(const TcNet *t, int node, int *leaves, int *nleaves, uint8_t *tt);

/* One pass of a program without id or link cells from power-on, input k in node leaves[k];
   cur[c] gets the node of cell c at the end. */
void tc_net_pass(TcNet *net, const Program *p, const uint32_t *in_cells, size_t n,
                 const int *leaves, int *cur);

#ifdef __cplusplus
}
#endif
#endif
