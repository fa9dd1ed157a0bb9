/* The reference machine on the host, for cuda_check only.

   `alpha check` is defined as "this engine against the reference machine" (src/check.c:52-113),
   so the check entry point needs the golden semantics next to the GPU engine: one byte per cell,
   one instruction at a time, every machine of the cube in lockstep, links followed to the
   neighbour across each dimension, id cells read from the machine number (src/ref.c:36-130).
   Nothing else in the engine runs programs on the host. */
#include <stdlib.h>
#include <string.h>

#include "ref_host.h"

int tc_ref_init(TcRef *r, const Program *p, unsigned machines)
{
    memset(r, 0, sizeof *r);
    r->p = p;
    r->machines = machines;
    r->mem = calloc((size_t)machines * p->ncells + 1, 1);
    r->rr = calloc(machines + 1, 1);
    r->addr = calloc(p->ncells + 1, sizeof *r->addr);
    r->mask = calloc(p->ncells + 1, sizeof *r->mask);
    if (!r->mem || !r->rr || !r->addr || !r->mask) {
        tc_ref_free(r);
        return 0;
    }
    for (uint32_t c = 0; c < p->ncells; c++)
        r->addr[c] = tc_program_resolve(p, c, &r->mask[c]);
    for (unsigned k = 0; k < machines; k++)
        r->mem[(size_t)k * p->ncells + CELL_ONE] = 1;
    return 1;
}

void tc_ref_free(TcRef *r)
{
    free(r->mem);
    free(r->rr);
    free(r->addr);
    free(r->mask);
    memset(r, 0, sizeof *r);
}

uint8_t tc_ref_get(const TcRef *r, unsigned k, uint32_t a)
{
    const Program *p = r->p;
    if (!p->special)
        return r->mem[(size_t)k * p->ncells + a];
    uint32_t c = r->addr[a];
    unsigned m = k ^ r->mask[a];
    if (p->special[c].kind == CK_ID)
        return (uint8_t)((m >> p->special[c].dim) & 1);
    return r->mem[(size_t)m * p->ncells + c];
}

/* One pass of every machine, instruction by instruction in lockstep. */
void tc_ref_tick(TcRef *r)
{
    const Program *p = r->p;
    for (size_t i = 0; i < p->len; i++) {
        Instr in = p->code[i];
        if (in.op == OP_NAND) {
            for (unsigned k = 0; k < r->machines; k++)
                r->rr[k] = (uint8_t)!(r->rr[k] & tc_ref_get(r, k, in.addr));
        } else if (!tc_program_readonly(p, in.addr)) {
            for (unsigned k = 0; k < r->machines; k++)
                r->mem[(size_t)k * p->ncells + in.addr] = r->rr[k];
        }
    }
}
