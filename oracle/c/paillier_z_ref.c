/*
 * CPU restatement of HEU's paillier_z hot path, for timing and as a second
 * checker.  TEST INFRASTRUCTURE ONLY: loaded by tests/ and by the CPU legs of
 * bench.py; the engine never links it.
 *
 * Follows (paths relative to the HEU project root):
 *   encrypt   heu/library/algorithms/paillier_zahlen/encryptor.cc:26-56
 *             with the fixed-base table of public_key.cc:28-40 (window 10,
 *             kExpUnitBits at public_key.cc:20)
 *   decrypt   heu/library/algorithms/paillier_zahlen/decryptor.cc:32-53
 *   add       heu/library/algorithms/paillier_zahlen/evaluator.cc:30-36
 *   mul       heu/library/algorithms/paillier_zahlen/evaluator.cc:99-123
 *   sum       heu/library/numpy/evaluator.cc:355-373
 *   bucket    heu/library/numpy/evaluator.cc:403-458 (FeatureWiseBucketSum)
 *   matmul    heu/library/numpy/evaluator.cc:208-292 (Mul + ReduceSum)
 * yacl's MontgomerySpace / BaseTable (not vendored) are restated with
 * 64-bit limbs and CIOS Montgomery multiplication; R = 2^(64*s) where s is the
 * number of 64-bit limbs of n^2 (the same radix as the engine's 32-bit R).
 * The per-ciphertext work runs on a pthread pool over contiguous chunks, as
 * yacl::parallel_for does for heu.numpy (numpy/encryptor.cc:24-39).
 */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

#define MAXS 96 /* 64-bit limbs of n^2 for 3072-bit keys */

typedef struct {
  int s;  /* 64-bit limbs of N = n^2 */
  uint64_t N[MAXS], np, R1[MAXS], R2[MAXS];
  uint64_t n[MAXS], nhalf[MAXS];
  int w, npos, rbits, rlimbs;
  uint64_t* table; /* npos * (2^w - 1) * s, Montgomery form */
  int has_sk;
  int h; /* 64-bit limbs of p (and q) */
  uint64_t P2[2][MAXS], np2[2], R2p[2][MAXS];
  uint64_t P[2][MAXS], np1[2], hR[2][MAXS], pinvqR[MAXS], inv2[2][MAXS];
  uint64_t e[2][MAXS];
  int ebits[2];
} pz_key;

/* ---------------- multi-limb helpers (s 64-bit limbs) ---------------- */
static uint64_t neg_inv64(uint64_t a) {
  uint64_t x = 1;
  for (int i = 0; i < 6; ++i) x *= 2 - a * x;
  return (uint64_t)0 - x;
}

static int cmp(const uint64_t* a, const uint64_t* b, int s) {
  for (int i = s - 1; i >= 0; --i)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

static uint64_t sub_n(uint64_t* r, const uint64_t* a, const uint64_t* b, int s) {
  uint64_t br = 0;
  for (int i = 0; i < s; ++i) {
    const uint64_t ai = a[i], bi = b[i];
    const uint64_t d = ai - bi - br;
    br = (ai < bi) || (ai == bi && br);
    r[i] = d;
  }
  return br;
}

static uint64_t add_n(uint64_t* r, const uint64_t* a, const uint64_t* b, int s) {
  u128 c = 0;
  for (int i = 0; i < s; ++i) {
    c += (u128)a[i] + b[i];
    r[i] = (uint64_t)c;
    c >>= 64;
  }
  return (uint64_t)c;
}

/* r = 2r mod m (r < m) */
static void dbl_mod(uint64_t* r, const uint64_t* m, int s) {
  uint64_t top = r[s - 1] >> 63;
  for (int i = s - 1; i > 0; --i) r[i] = (r[i] << 1) | (r[i - 1] >> 63);
  r[0] <<= 1;
  if (top || cmp(r, m, s) >= 0) sub_n(r, r, m, s);
}

/* CIOS Montgomery multiplication: r = a*b*R^-1 mod m, a < R, b < m. */
static void mont_mul(uint64_t* r, const uint64_t* a, const uint64_t* b, const uint64_t* m, uint64_t np, int s) {
  uint64_t t[MAXS + 2];
  memset(t, 0, sizeof(uint64_t) * (s + 2));
  for (int i = 0; i < s; ++i) {
    u128 c = 0;
    const uint64_t bi = b[i];
    for (int j = 0; j < s; ++j) {
      c += (u128)a[j] * bi + t[j];
      t[j] = (uint64_t)c;
      c >>= 64;
    }
    c += t[s];
    t[s] = (uint64_t)c;
    t[s + 1] = (uint64_t)(c >> 64);
    const uint64_t mq = t[0] * np;
    c = ((u128)mq * m[0] + t[0]) >> 64;
    for (int j = 1; j < s; ++j) {
      c += (u128)mq * m[j] + t[j];
      t[j - 1] = (uint64_t)c;
      c >>= 64;
    }
    c += t[s];
    t[s - 1] = (uint64_t)c;
    t[s] = t[s + 1] + (uint64_t)(c >> 64);
  }
  if (t[s] || cmp(t, m, s) >= 0) sub_n(t, t, m, s);
  memcpy(r, t, sizeof(uint64_t) * s);
}

static void one_limbs(uint64_t* x, int s) {
  memset(x, 0, sizeof(uint64_t) * s);
  x[0] = 1;
}

/* R^k mod m by doubling (setup only) */
static void pow2_mod(uint64_t* r, int bits, const uint64_t* m, int s) {
  one_limbs(r, s);
  for (int i = 0; i < bits; ++i) dbl_mod(r, m, s);
}

/* Binary extended Euclid: r = a^-1 mod m (m odd).  Returns 0 if not invertible. */
static int inv_mod(uint64_t* r, const uint64_t* a, const uint64_t* m, int s) {
  uint64_t u[MAXS], v[MAXS], x1[MAXS], x2[MAXS], z[MAXS];
  memcpy(u, a, 8 * s);
  memcpy(v, m, 8 * s);
  one_limbs(x1, s);
  memset(x2, 0, 8 * s);
  memset(z, 0, 8 * s);
  one_limbs(r, s);
  for (;;) {
    if (cmp(u, z, s) == 0) return 0;
    uint64_t one[MAXS];
    one_limbs(one, s);
    if (cmp(u, one, s) == 0) {
      memcpy(r, x1, 8 * s);
      return 1;
    }
    if (cmp(v, one, s) == 0) {
      memcpy(r, x2, 8 * s);
      return 1;
    }
    while (!(u[0] & 1)) {
      for (int i = 0; i < s - 1; ++i) u[i] = (u[i] >> 1) | (u[i + 1] << 63);
      u[s - 1] >>= 1;
      uint64_t c = 0;
      if (x1[0] & 1) c = add_n(x1, x1, m, s);
      for (int i = 0; i < s - 1; ++i) x1[i] = (x1[i] >> 1) | (x1[i + 1] << 63);
      x1[s - 1] = (x1[s - 1] >> 1) | (c << 63);
    }
    while (!(v[0] & 1)) {
      for (int i = 0; i < s - 1; ++i) v[i] = (v[i] >> 1) | (v[i + 1] << 63);
      v[s - 1] >>= 1;
      uint64_t c = 0;
      if (x2[0] & 1) c = add_n(x2, x2, m, s);
      for (int i = 0; i < s - 1; ++i) x2[i] = (x2[i] >> 1) | (x2[i + 1] << 63);
      x2[s - 1] = (x2[s - 1] >> 1) | (c << 63);
    }
    if (cmp(u, v, s) >= 0) {
      sub_n(u, u, v, s);
      if (sub_n(x1, x1, x2, s)) add_n(x1, x1, m, s);
    } else {
      sub_n(v, v, u, s);
      if (sub_n(x2, x2, x1, s)) add_n(x2, x2, m, s);
    }
  }
}

/* Montgomery-space exponentiation by left-to-right sliding windows. */
static void mont_pow(uint64_t* r, const uint64_t* xm, const uint64_t* e, int ebits, const uint64_t* m,
                     uint64_t np, const uint64_t* one_m, int s, int w) {
  uint64_t tab[32][MAXS], x2[MAXS], acc[MAXS];
  const int nt = 1 << (w - 1);
  memcpy(tab[0], xm, 8 * s);
  mont_mul(x2, xm, xm, m, np, s);
  for (int i = 1; i < nt; ++i) mont_mul(tab[i], tab[i - 1], x2, m, np, s);
  memcpy(acc, one_m, 8 * s);
  int i = ebits - 1;
  int first = 1;
  while (i >= 0) {
    if (!((e[i / 64] >> (i % 64)) & 1)) {
      if (!first) mont_mul(acc, acc, acc, m, np, s);
      --i;
      continue;
    }
    int j = i - w + 1 < 0 ? 0 : i - w + 1;
    while (!((e[j / 64] >> (j % 64)) & 1)) ++j;
    uint32_t val = 0;
    for (int b = i; b >= j; --b) val = (val << 1) | (uint32_t)((e[b / 64] >> (b % 64)) & 1);
    if (first) {
      memcpy(acc, tab[(val - 1) >> 1], 8 * s);
      first = 0;
    } else {
      for (int t = 0; t < i - j + 1; ++t) mont_mul(acc, acc, acc, m, np, s);
      mont_mul(acc, acc, tab[(val - 1) >> 1], m, np, s);
    }
    i = j - 1;
  }
  memcpy(r, acc, 8 * s);
}

/* ---------------- key setup ---------------- */
static int bitlen_n(const uint64_t* x, int s) {
  for (int i = s - 1; i >= 0; --i)
    if (x[i]) return 64 * i + 64 - __builtin_clzll(x[i]);
  return 0;
}

/* All arrays little-endian 64-bit limbs: n (s/2), hs (s), p q (s/4),
 * hp hq pinvq (s/4), pinv2 qinv2 = p^-1, q^-1 mod 2^(64*s/4) (s/4). */
pz_key* pz_key_create(int key_bits, const uint64_t* n, const uint64_t* hs, const uint64_t* p, const uint64_t* q,
                      const uint64_t* hp, const uint64_t* hq, const uint64_t* pinvq, const uint64_t* pinv2,
                      const uint64_t* qinv2, int w) {
  pz_key* k = (pz_key*)calloc(1, sizeof(pz_key));
  if (!k) return NULL;
  const int s = key_bits / 32;
  k->s = s;
  memcpy(k->n, n, 8 * (s / 2));
  /* N = n*n */
  for (int i = 0; i < s / 2; ++i) {
    u128 c = 0;
    for (int j = 0; j < s / 2; ++j) {
      c += (u128)n[i] * n[j] + k->N[i + j];
      k->N[i + j] = (uint64_t)c;
      c >>= 64;
    }
    k->N[i + s / 2] = (uint64_t)c;
  }
  k->np = neg_inv64(k->N[0]);
  pow2_mod(k->R1, 64 * s, k->N, s);
  memcpy(k->R2, k->R1, 8 * s);
  for (int i = 0; i < 64 * s; ++i) dbl_mod(k->R2, k->N, s);
  for (int i = 0; i < s / 2; ++i) k->nhalf[i] = (n[i] >> 1) | (i + 1 < s / 2 ? n[i + 1] << 63 : 0);
  const int kbits = bitlen_n(n, s / 2);
  k->rbits = kbits / 2;
  k->rlimbs = key_bits / 128; /* 64-bit limbs of r */
  k->w = w;
  k->npos = (k->rbits + w - 1) / w;
  const size_t ent = ((size_t)1 << w) - 1;
  k->table = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)k->npos * ent * s);
  if (!k->table) {
    free(k);
    return NULL;
  }
  /* public_key.cc:36-39: base table of h_s powers */
  uint64_t g[MAXS], hsv[MAXS];
  memset(hsv, 0, sizeof(hsv));
  memcpy(hsv, hs, 8 * s);
  mont_mul(g, hsv, k->R2, k->N, k->np, s);
  for (int pos = 0; pos < k->npos; ++pos) {
    uint64_t* row = k->table + (size_t)pos * ent * s;
    memcpy(row, g, 8 * s);
    for (size_t d = 2; d <= ent; ++d) mont_mul(row + (d - 1) * s, row + (d - 2) * s, g, k->N, k->np, s);
    for (int t = 0; t < w; ++t) mont_mul(g, g, g, k->N, k->np, s);
  }
  if (p && q) {
    k->has_sk = 1;
    const int h = s / 4, sp = s / 2;
    k->h = h;
    const uint64_t* pr[2] = {p, q};
    const uint64_t* hh[2] = {hp, hq};
    const uint64_t* iv[2] = {pinv2, qinv2};
    for (int sd = 0; sd < 2; ++sd) {
      memcpy(k->P[sd], pr[sd], 8 * h);
      for (int i = 0; i < h; ++i) {
        u128 c = 0;
        for (int j = 0; j < h; ++j) {
          c += (u128)pr[sd][i] * pr[sd][j] + k->P2[sd][i + j];
          k->P2[sd][i + j] = (uint64_t)c;
          c >>= 64;
        }
        k->P2[sd][i + h] = (uint64_t)c;
      }
      k->np2[sd] = neg_inv64(k->P2[sd][0]);
      pow2_mod(k->R2p[sd], 2 * 64 * sp, k->P2[sd], sp);
      k->np1[sd] = neg_inv64(pr[sd][0]);
      uint64_t r2[MAXS];
      pow2_mod(r2, 2 * 64 * h, pr[sd], h);
      uint64_t hv[MAXS];
      memset(hv, 0, sizeof(hv));
      memcpy(hv, hh[sd], 8 * h);
      mont_mul(k->hR[sd], hv, r2, pr[sd], k->np1[sd], h); /* hp*R mod p */
      memcpy(k->inv2[sd], iv[sd], 8 * h);
      memcpy(k->e[sd], pr[sd], 8 * h);
      k->e[sd][0] -= 1; /* p - 1 (p odd) */
      k->ebits[sd] = bitlen_n(k->e[sd], h);
      if (sd == 1) {
        uint64_t pv[MAXS];
        memset(pv, 0, sizeof(pv));
        memcpy(pv, pinvq, 8 * h);
        mont_mul(k->pinvqR, pv, r2, pr[1], k->np1[1], h);
      }
    }
  }
  return k;
}

void pz_key_free(pz_key* k) {
  if (k) {
    free(k->table);
    free(k);
  }
}

/* ---------------- per-ciphertext operations ---------------- */
static void enc_one(const pz_key* k, int64_t m, const uint64_t* r, uint64_t* out) {
  const int s = k->s;
  /* gm = 1 + n*m mod n^2 (encryptor.cc:44) */
  uint64_t gm[MAXS], t[MAXS];
  memset(t, 0, sizeof(t));
  const uint64_t mag = m < 0 ? (uint64_t)0 - (uint64_t)m : (uint64_t)m;
  u128 c = 0;
  for (int i = 0; i < s / 2; ++i) {
    c += (u128)k->n[i] * mag;
    t[i] = (uint64_t)c;
    c >>= 64;
  }
  t[s / 2] = (uint64_t)c;
  if (m < 0 && mag) {
    sub_n(gm, k->N, t, s);
  } else {
    memcpy(gm, t, 8 * s);
  }
  /* + 1 */
  for (int i = 0; i < s; ++i)
    if (++gm[i]) break;
  if (cmp(gm, k->N, s) >= 0) sub_n(gm, gm, k->N, s);
  mont_mul(gm, gm, k->R2, k->N, k->np, s); /* MapIntoMSpace */
  /* GetRn: h_s^r from the table (encryptor.cc:26-31) */
  const size_t ent = ((size_t)1 << k->w) - 1;
  uint64_t acc[MAXS];
  memcpy(acc, k->R1, 8 * s);
  for (int pos = 0; pos < k->npos; ++pos) {
    const int off = pos * k->w;
    const int li = off / 64, sh = off % 64;
    u128 v = r[li];
    if (li + 1 < k->rlimbs) v |= (u128)r[li + 1] << 64;
    int wbits = k->w;
    if (k->rbits - off < wbits) wbits = k->rbits - off;
    const uint64_t dg = (uint64_t)(v >> sh) & (((uint64_t)1 << wbits) - 1);
    if (dg) mont_mul(acc, acc, k->table + ((size_t)pos * ent + dg - 1) * s, k->N, k->np, s);
  }
  mont_mul(out, gm, acc, k->N, k->np, s);
}

static int dec_one(const pz_key* k, const uint64_t* ct, int64_t* out, uint8_t* ovf) {
  const int s = k->s, sp = s / 2, h = s / 4;
  uint64_t c[MAXS], one[MAXS];
  one_limbs(one, s);
  mont_mul(c, ct, one, k->N, k->np, s); /* MapBackToZSpace */
  uint64_t mpq[2][MAXS];
  for (int sd = 0; sd < 2; ++sd) {
    /* c mod p^2: c = hi*2^(64 sp) + lo; Montgomery form = REDC(c)*R2p ... via mont_mul */
    uint64_t lo[MAXS], hi[MAXS], xm[MAXS], tmp[MAXS], onep[MAXS], y[MAXS];
    memcpy(lo, c, 8 * sp);
    memcpy(hi, c + sp, 8 * sp);
    /* x = (hi*Rp + lo) mod p^2; Montgomery form x*Rp = MM(hi, R2p)*Rp.. computed as
       MM(lo, R2p) + MM(MM(hi, R2p), R2p) */
    mont_mul(xm, lo, k->R2p[sd], k->P2[sd], k->np2[sd], sp);
    mont_mul(tmp, hi, k->R2p[sd], k->P2[sd], k->np2[sd], sp);
    mont_mul(tmp, tmp, k->R2p[sd], k->P2[sd], k->np2[sd], sp);
    if (add_n(xm, xm, tmp, sp) || cmp(xm, k->P2[sd], sp) >= 0) sub_n(xm, xm, k->P2[sd], sp);
    uint64_t onem[MAXS];
    one_limbs(onep, sp);
    mont_mul(onem, onep, k->R2p[sd], k->P2[sd], k->np2[sd], sp);
    /* c^(p-1) mod p^2 (decryptor.cc:38) */
    mont_pow(y, xm, k->e[sd], k->ebits[sd], k->P2[sd], k->np2[sd], onem, sp, 5);
    mont_mul(y, y, onep, k->P2[sd], k->np2[sd], sp);
    /* L = (y - 1)/p exactly, via p^-1 mod 2^(64h) */
    uint64_t t1[MAXS], L[MAXS];
    memcpy(t1, y, 8 * h);
    for (int i = 0; i < h; ++i)
      if (t1[i]--) break;
    memset(L, 0, sizeof(L));
    for (int a = 0; a < h; ++a) {
      u128 cc = 0;
      for (int b = 0; a + b < h; ++b) {
        cc += (u128)t1[a] * k->inv2[sd][b] + L[a + b];
        L[a + b] = (uint64_t)cc;
        cc >>= 64;
      }
    }
    /* * hp mod p (decryptor.cc:39) */
    mont_mul(mpq[sd], L, k->hR[sd], k->P[sd], k->np1[sd], h);
  }
  /* CRT (decryptor.cc:44-47) */
  uint64_t mpq_q[MAXS], d[MAXS], hh[MAXS], m[MAXS];
  if (sub_n(mpq_q, mpq[0], k->P[1], h)) memcpy(mpq_q, mpq[0], 8 * h);
  if (sub_n(d, mpq[1], mpq_q, h)) add_n(d, d, k->P[1], h);
  mont_mul(hh, d, k->pinvqR, k->P[1], k->np1[1], h);
  memset(m, 0, sizeof(m));
  memcpy(m, mpq[0], 8 * h);
  for (int a = 0; a < h; ++a) {
    u128 cc = 0;
    for (int b = 0; b < h; ++b) {
      cc += (u128)k->P[0][a] * hh[b] + m[a + b];
      m[a + b] = (uint64_t)cc;
      cc >>= 64;
    }
    for (int j = a + h; cc && j < sp; ++j) {
      cc += m[j];
      m[j] = (uint64_t)cc;
      cc >>= 64;
    }
  }
  /* m > n/2 => m - n (decryptor.cc:49-52) */
  int neg = cmp(m, k->nhalf, sp) > 0;
  if (neg) sub_n(m, k->n, m, sp);
  int fits = 1;
  for (int i = 1; i < sp; ++i) fits &= (m[i] == 0);
  if (neg) {
    fits &= m[0] <= ((uint64_t)1 << 63);
    *out = (int64_t)((uint64_t)0 - m[0]);
  } else {
    fits &= m[0] < ((uint64_t)1 << 63);
    *out = (int64_t)m[0];
  }
  if (ovf) *ovf = fits ? 0 : 1;
  return 0;
}

static int mul_one(const pz_key* k, const uint64_t* ct, int64_t kk, uint64_t* out) {
  const int s = k->s;
  if (kk == 0) { /* evaluator.cc:105-106 */
    memcpy(out, k->R1, 8 * s);
    return 0;
  }
  const uint64_t e = kk < 0 ? (uint64_t)0 - (uint64_t)kk : (uint64_t)kk;
  uint64_t acc[MAXS];
  mont_pow(acc, ct, &e, 64 - __builtin_clzll(e), k->N, k->np, k->R1, s, 4);
  if (kk < 0) {
    /* (c^|k|)^-1 in Montgomery form: inv(X R) = X^-1 R^-1; * R^3 via two R2 mults */
    uint64_t z[MAXS];
    if (!inv_mod(z, acc, k->N, s)) return 1;
    mont_mul(z, z, k->R2, k->N, k->np, s);
    mont_mul(acc, z, k->R2, k->N, k->np, s);
  }
  memcpy(out, acc, 8 * s);
  return 0;
}

/* ---------------- thread pool over chunks ---------------- */
typedef struct {
  const pz_key* k;
  int op;
  const void* a;
  const void* b;
  void* out;
  void* out2;
  size_t beg, end;
  int err;
  size_t d0, d1, d2; /* shape of the reductions (rows/M, F/K, B/N) */
} job_t;

static void* worker(void* arg) {
  job_t* j = (job_t*)arg;
  const pz_key* k = j->k;
  const int s = k->s;
  for (size_t i = j->beg; i < j->end; ++i) {
    switch (j->op) {
      case 0:
        enc_one(k, ((const int64_t*)j->a)[i], (const uint64_t*)j->b + i * k->rlimbs, (uint64_t*)j->out + i * s);
        break;
      case 1:
        dec_one(k, (const uint64_t*)j->a + i * s, (int64_t*)j->out + i, j->out2 ? (uint8_t*)j->out2 + i : NULL);
        break;
      case 2:
        mont_mul((uint64_t*)j->out + i * s, (const uint64_t*)j->a + i * s, (const uint64_t*)j->b + i * s, k->N,
                 k->np, s);
        break;
      case 3:
        if (mul_one(k, (const uint64_t*)j->a + i * s, ((const int64_t*)j->b)[i], (uint64_t*)j->out + i * s))
          j->err = 1;
        break;
      case 4: { /* bucket sums of feature i: buckets start at the identity (GetZero) */
        const size_t rows = j->d0, F = j->d1, B = j->d2;
        const uint64_t* x = (const uint64_t*)j->a;
        const uint8_t* om = (const uint8_t*)j->b;
        uint64_t* out = (uint64_t*)j->out + i * B * s;
        for (size_t b = 0; b < B; ++b) memcpy(out + b * s, k->R1, 8 * s);
        for (size_t r = 0; r < rows; ++r) {
          const size_t b = om[r * F + i];
          if (b >= B) {
            j->err = 1;
            continue;
          }
          mont_mul(out + b * s, out + b * s, x + r * s, k->N, k->np, s);
        }
        break;
      }
      case 5: { /* output element i of MatMul: prod_kk Mul(x(row, kk), y(kk, col)) */
        const size_t K = j->d1, N = j->d2, row = i / N, col = i % N;
        const uint64_t* x = (const uint64_t*)j->a + row * K * s;
        const int64_t* y = (const int64_t*)j->b;
        uint64_t acc[MAXS], t[MAXS];
        if (mul_one(k, x, y[col], acc)) j->err = 1;
        for (size_t kk = 1; kk < K; ++kk) {
          if (mul_one(k, x + kk * s, y[kk * N + col], t)) j->err = 1;
          mont_mul(acc, acc, t, k->N, k->np, s);
        }
        memcpy((uint64_t*)j->out + i * s, acc, 8 * s);
        break;
      }
      case 6: { /* partial product of this thread's range (numpy Sum) */
        if (i == j->beg) memcpy(j->out2, (const uint64_t*)j->a + i * s, 8 * s);
        else mont_mul((uint64_t*)j->out2, (const uint64_t*)j->out2, (const uint64_t*)j->a + i * s, k->N, k->np, s);
        break;
      }
    }
  }
  return NULL;
}

static int run_shaped(const pz_key* k, int op, const void* a, const void* b, void* out, void* out2, size_t count,
                      int threads, size_t d0, size_t d1, size_t d2, uint64_t* partials) {
  if (threads < 1) threads = 1;
  if ((size_t)threads > count) threads = count ? (int)count : 1;
  pthread_t th[256];
  job_t jobs[256];
  if (threads > 256) threads = 256;
  for (int t = 0; t < threads; ++t) {
    jobs[t] = (job_t){k, op, a, b, out, partials ? partials + (size_t)t * k->s : out2,
                      count * t / threads, count * (t + 1) / threads, 0, d0, d1, d2};
    pthread_create(&th[t], NULL, worker, &jobs[t]);
  }
  int err = 0;
  for (int t = 0; t < threads; ++t) {
    pthread_join(th[t], NULL);
    err |= jobs[t].err;
  }
  return err;
}

static int run(const pz_key* k, int op, const void* a, const void* b, void* out, void* out2, size_t count,
               int threads) {
  return run_shaped(k, op, a, b, out, out2, count, threads, 0, 0, 0, NULL);
}

int pz_encrypt(const pz_key* k, const int64_t* m, const uint64_t* r, uint64_t* out, size_t count, int threads) {
  return run(k, 0, m, r, out, NULL, count, threads);
}
int pz_decrypt(const pz_key* k, const uint64_t* ct, int64_t* out, uint8_t* ovf, size_t count, int threads) {
  if (!k->has_sk) return 2;
  return run(k, 1, ct, NULL, out, ovf, count, threads);
}
int pz_add(const pz_key* k, const uint64_t* a, const uint64_t* b, uint64_t* out, size_t count, int threads) {
  return run(k, 2, a, b, out, NULL, count, threads);
}
int pz_mul(const pz_key* k, const uint64_t* a, const int64_t* kk, uint64_t* out, size_t count, int threads) {
  return run(k, 3, a, kk, out, NULL, count, threads);
}
/* product of all ciphertexts (numpy Sum), single thread */
int pz_sum(const pz_key* k, const uint64_t* a, size_t count, uint64_t* out) {
  const int s = k->s;
  if (count == 0) return 1;
  uint64_t acc[MAXS];
  memcpy(acc, a, 8 * s);
  for (size_t i = 1; i < count; ++i) mont_mul(acc, acc, a + i * s, k->N, k->np, s);
  memcpy(out, acc, 8 * s);
  return 0;
}

/* numpy Sum over a thread pool: one partial product per thread, combined in
 * order (parallel_reduce of numpy/evaluator.cc:355-373) */
int pz_sum_mt(const pz_key* k, const uint64_t* a, size_t count, uint64_t* out, int threads) {
  const int s = k->s;
  if (count == 0) return 1;
  if (threads < 1) threads = 1;
  if ((size_t)threads > count) threads = (int)count;
  if (threads > 256) threads = 256;
  uint64_t* part = (uint64_t*)malloc((size_t)threads * s * 8);
  if (!part) return 3;
  const int err = run_shaped(k, 6, a, NULL, NULL, NULL, count, threads, 0, 0, 0, part);
  memcpy(out, part, 8 * s);
  for (int t = 1; t < threads; ++t) mont_mul(out, out, part + (size_t)t * s, k->N, k->np, s);
  free(part);
  return err;
}

/* FeatureWiseBucketSum of one ciphertext column x (rows) with order map om
 * (rows x F, bin ids < B): out[f * B + b] = prod of x[r] with om[r, f] == b,
 * the identity for empty buckets; features over the thread pool */
int pz_bucket_sum(const pz_key* k, const uint64_t* x, size_t rows, const uint8_t* om, size_t F, size_t B,
                  uint64_t* out, int threads) {
  return run_shaped(k, 4, x, om, out, NULL, F, threads, rows, F, B, NULL);
}

/* MatMul out(i, j) = prod_kk Mul(x(i, kk), y(kk, j)) for x M x K ciphertexts
 * and y K x N int64 scalars; output elements over the thread pool */
int pz_matmul(const pz_key* k, const uint64_t* x, size_t M, size_t K, const int64_t* y, size_t N, uint64_t* out,
              int threads) {
  return run_shaped(k, 5, x, y, out, NULL, M * N, threads, M, K, N, NULL);
}
