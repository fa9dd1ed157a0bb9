/* Host stand-ins for the three CUDA intrinsics the generated per-word function uses, so the tests
   can compile the engine's generated CUDA C with gcc and check the code generator on a CPU.
   Only the tests include this; the engine never runs generated code on the host. */
#ifndef TC_HOST_EMULATION_H
#define TC_HOST_EMULATION_H
#define TC_HOST_EMULATION 1

static inline unsigned __byte_perm(unsigned x, unsigned y, unsigned s)
{
    unsigned long long v = (unsigned long long)y << 32 | x, r = 0;
    for (int i = 0; i < 4; i++)
        r |= ((v >> (8 * ((s >> (4 * i)) & 7))) & 0xffull) << (8 * i);
    return (unsigned)r;
}

static inline unsigned long long __brevll(unsigned long long x)
{
    unsigned long long r = 0;
    for (int i = 0; i < 64; i++)
        r |= ((x >> i) & 1ull) << (63 - i);
    return r;
}

#endif
