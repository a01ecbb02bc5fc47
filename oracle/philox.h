/*
 * Philox4x32-10 counter-based generator (Salmon, Moraes, Dror & Shaw,
 * "Parallel random numbers: as easy as 1, 2, 3", SC'11), restated from the
 * published algorithm for the CPU oracle.  Test infrastructure only.
 *
 * Packet streams: key = (seed_lo ^ iter*0x9E3779B9, seed_hi), counter =
 * (block, 0, pid_lo, pid_hi); each block yields four 32-bit draws, turned
 * into doubles in (0,1) by (u + 0.5) * 2^-32.  This replaces the L'Ecuyer-
 * Cote stream of the reference (random.f90:99-118, ecuyer_cote_mod.f90:252)
 * so that every packet's draws depend only on (seed, iter, packet id).
 */
#ifndef HC3D_ORACLE_PHILOX_H
#define HC3D_ORACLE_PHILOX_H
#include <math.h>
#include <stdint.h>

#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0;
    uint32_t n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += PHILOX_W0; k1 += PHILOX_W1;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

typedef struct orc_rng {
  uint32_t key[2];
  uint32_t ctr[4];
  uint32_t buf[4];
  int left;
  /* injected uniforms (trace harness); NULL for the counter stream */
  const double *inj;
  int ninj, pos;
  int exhausted;
} orc_rng;

static inline void orc_rng_init(orc_rng *r, uint64_t seed, int iter, int64_t pid) {
  r->key[0] = (uint32_t)seed ^ ((uint32_t)iter * PHILOX_W0);
  r->key[1] = (uint32_t)(seed >> 32);
  r->ctr[0] = 0; r->ctr[1] = 0;
  r->ctr[2] = (uint32_t)(uint64_t)pid;
  r->ctr[3] = (uint32_t)((uint64_t)pid >> 32);
  r->left = 0;
  r->inj = 0; r->ninj = 0; r->pos = 0; r->exhausted = 0;
}

static inline double orc_ran(orc_rng *r) {
  if (r->inj) {
    if (r->pos < r->ninj) return r->inj[r->pos++];
    /* past the end of the injected list: frac(0.5 + k (sqrt(5) - 1) / 2),
     * as the device continues, so that rejection loops still end */
    r->exhausted = 1;
    double v = 0.5 + (double)(r->pos++ - r->ninj) * 0.6180339887498949;
    return v - floor(v);
  }
  if (r->left == 0) {
    orc_philox4x32_10(r->ctr, r->key, r->buf);
    r->ctr[0]++;
    r->left = 4;
  }
  uint32_t u = r->buf[4 - r->left];
  r->left--;
  return ((double)u + 0.5) * (1.0 / 4294967296.0);
}

#endif
