/*
 * rsc_populate.h -- internal: the generator behind rsc_populate_host and
 * rsc_populate_upload (rsc_populate.cpp).
 */
#ifndef SIMRADAR_GB300_RSC_POPULATE_H
#define SIMRADAR_GB300_RSC_POPULATE_H

#include <stddef.h>
#include <stdint.h>

#include "../../include/rsc.h"

namespace rscpop {

/* glibc rand(): the last 34 values of the lagged-Fibonacci sequence */
struct RandState {
    uint32_t r[34];
    int pos;   /* i mod 34 of the next value */
};

void rand_seed(RandState *s, uint32_t seed);
int32_t rand_next(RandState *s);

/* RS_populate's draws in slot order for one worker whose type ranges follow
 * one another from slot 0 (origins[k] = counts[0] + ... + counts[k-1]). */
struct Generator {
    rsc_populate_args a;
    RandState main_rs, dsd_rs;
    size_t next_slot = 0, total = 0;
    int init(const rsc_populate_args *args, const char **why);
    /* the next n slots: pos, aux and rnd (4 values per slot) */
    void fill(size_t n, float *pos4, float *aux4, uint32_t *rnd4, uint32_t *dsd_pop);
};

}  // namespace rscpop

#endif
