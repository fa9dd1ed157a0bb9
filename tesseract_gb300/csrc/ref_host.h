/* The host reference machine used by cuda_check (ref_host.c). */
#ifndef TC_REF_HOST_H
#define TC_REF_HOST_H

#include "tc_host.h"

typedef struct {
    const Program *p;
    unsigned       machines;
    uint8_t       *mem;   /* machines x ncells bytes */
    uint8_t       *rr;
    uint32_t      *addr;  /* per cell: the cell a read really reaches */
    unsigned      *mask;  /* and the machines it crosses */
} TcRef;

int     tc_ref_init(TcRef *r, const Program *p, unsigned machines);
void    tc_ref_free(TcRef *r);
uint8_t tc_ref_get(const TcRef *r, unsigned k, uint32_t a);
void    tc_ref_tick(TcRef *r);

#endif
