/* Test-only stand-in for the GSL random-number symbols the reference's theory vpf calls
 * (theory/vpf/countspheres_impl.c.src:189-195, 287-289, 422): gsl_rng_mt19937 only.  GSL is not
 * installed here; this header lets oracle/build_ref.py compile the reference sources unchanged,
 * as the checker.
 *
 * The generator is restated from the published MT19937 (Matsumoto & Nishimura 1998) with the
 * 2002 initialisation that GSL uses: seed 0 is replaced by 4357, state[0] = seed, state[i] =
 * 1812433253 * (state[i-1] ^ (state[i-1] >> 30)) + i; gsl_rng_uniform returns the next 32-bit
 * output divided by 2^32.  Nothing in the product includes this file. */
#ifndef CF_GSL_SHIM_RNG_H
#define CF_GSL_SHIM_RNG_H
#include <stdint.h>
#include <stdlib.h>

typedef struct {
    const char *name;
} gsl_rng_type;

typedef struct {
    uint32_t s[624];
    int next; /* next state word to temper; 624 = regenerate first */
} gsl_rng;

static const gsl_rng_type cf_shim_rng_mt19937 = {"mt19937"};
#define gsl_rng_mt19937 (&cf_shim_rng_mt19937)

static inline void gsl_rng_set(gsl_rng *r, unsigned long int seed)
{
    uint32_t v = (uint32_t)(seed == 0 ? 4357ul : seed);
    r->s[0] = v;
    for (int i = 1; i < 624; i++) {
        v = 1812433253u * (v ^ (v >> 30)) + (uint32_t)i;
        r->s[i] = v;
    }
    r->next = 624;
}

static inline gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
    (void)T;
    gsl_rng *r = (gsl_rng *)malloc(sizeof(gsl_rng));
    if (r) gsl_rng_set(r, 0); /* GSL seeds a new generator with its default seed */
    return r;
}

static inline void gsl_rng_free(gsl_rng *r) { free(r); }

static inline uint32_t cf_shim_mt_next(gsl_rng *r)
{
    if (r->next >= 624) {
        for (int k = 0; k < 624; k++) {
            const uint32_t hi = r->s[k] & 0x80000000u, lo = r->s[k + 1 < 624 ? k + 1 : 0] & 0x7fffffffu;
            const uint32_t y = hi | lo;
            const uint32_t mag = (y & 1u) ? 0x9908b0dfu : 0u;
            r->s[k] = r->s[k + 397 < 624 ? k + 397 : k + 397 - 624] ^ (y >> 1) ^ mag;
        }
        r->next = 0;
    }
    uint32_t t = r->s[r->next++];
    t ^= t >> 11;
    t ^= (t << 7) & 0x9d2c5680u;
    t ^= (t << 15) & 0xefc60000u;
    t ^= t >> 18;
    return t;
}

static inline double gsl_rng_uniform(const gsl_rng *r) { return cf_shim_mt_next((gsl_rng *)r) / 4294967296.0; }
#endif
