/*
 * ngenic_oracle.h -- CPU restatement of generate_ngeniclike_grf and of the RANLUX (ranlxd1)
 * generator it uses.  TEST INFRASTRUCTURE ONLY; parity with libgsl unpinned (see the .c file).
 */
#ifndef NGENIC_ORACLE_H
#define NGENIC_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

struct orc_ranlxd {
    uint64_t x[12];  /* 48-bit words */
    int carry;
    int i;           /* next word to overwrite (the oldest) */
    int left;        /* words of the current block not yet delivered */
};

void orc_ranlxd1_set(struct orc_ranlxd *r, unsigned long seed);
double orc_ranlxd1_uniform(struct orc_ranlxd *r);
void orc_ngenic_seedtable(int N, unsigned long seed, unsigned int *table);
/* fbox: N x N x (N/2+1) complex, interleaved (re, im) doubles */
int orc_ngeniclike_grf(int N, double boxlen, unsigned long seed, double *fbox);

#ifdef __cplusplus
}
#endif
#endif
