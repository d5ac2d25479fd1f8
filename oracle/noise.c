/* Oracle restatement of the engine's Fourier-space noise stream, in C
 * (TEST INFRASTRUCTURE ONLY: loaded by oracle/philox.py for tests/, the smoke check and
 * the CPU-baseline leg of bench.py; never part of the library).
 *
 * Same definition as oracle/philox.py::fourier_noise, which documents it: counter-based
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) with key (seed mod 2^32, seed >> 32)
 * and counter (c, step, field_id, 0); Box-Muller on word pairs; the folded line-axis
 * counters of the modes 0 < kx < sx/2, the canonical pair member on the kx = 0 and
 * kx = sx/2 planes, Hermitian partners for kx > sx/2.  It replaces the reference's
 * time-seeded cuRAND normals + forward FFT (src/field.cpp:300-316), whose realisation
 * cannot be reproduced.  Output: the full reference-layout spectrum [kz][ky][kx] as
 * interleaved (re, im) doubles.  The numpy version is kept as the cross-check. */
#include <math.h>
#include <stddef.h>
#include <stdint.h>

static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)c[0] * 0xD2511F53u;
    const uint64_t p1 = (uint64_t)c[2] * 0xCD9E8D57u;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

/* u1 = ((a >> 8) + 1) 2^-24 in (0, 1], u2 = (b >> 8) 2^-24 in [0, 1),
 * g1 + i g2 = sqrt(-2 ln u1) exp(2 pi i (u2 - 1/2)) */
static void normal_pair(uint32_t a, uint32_t b, double* g1, double* g2) {
  const double u1 = ((double)(a >> 8) + 1.0) * (1.0 / 16777216.0);
  const double u2 = (double)(b >> 8) * (1.0 / 16777216.0);
  const double r = sqrt(-2.0 * log(u1));
  const double ang = 2.0 * 3.14159265358979323846 * (u2 - 0.5);
  *g1 = r * cos(ang);
  *g2 = r * sin(ang);
}

/* the mode (kx, ky, kz) with kx <= sx/2 */
static void mode(int sx, int sy, int sz, uint32_t k0, uint32_t k1, uint32_t step, uint32_t fid, int kx, int ky,
                 int kz, double* re, double* im) {
  const double N = (double)sx * sy * sz;
  const double half = sqrt(N / 2.0);
  uint32_t c[4];
  double g1, g2;
  if (kx > 0 && 2 * kx < sx) {
    const int Lt = sz > 1 ? sz : (sy > 1 ? sy : 1);
    int t = sz > 1 ? kz : ky;
    int upper = 0;
    if (Lt > 1 && t >= Lt / 2) {
      upper = 1;
      t -= Lt / 2;
    }
    const int fkz = sz > 1 ? t : kz, fky = sz > 1 ? ky : t;
    c[0] = (uint32_t)(((uint64_t)fkz * sy + fky) * sx + kx);
    c[1] = step;
    c[2] = fid;
    c[3] = 0u;
    philox4x32_10(c, k0, k1);
    if (upper) normal_pair(c[2], c[3], &g1, &g2);
    else normal_pair(c[0], c[1], &g1, &g2);
    *re = half * g1;
    *im = half * g2;
    return;
  }
  const uint64_t lin = ((uint64_t)kz * sy + ky) * sx + kx;
  const uint64_t plin = ((uint64_t)((sz - kz) % sz) * sy + (uint64_t)((sy - ky) % sy)) * sx + kx;
  c[0] = (uint32_t)(lin < plin ? lin : plin);
  c[1] = step;
  c[2] = fid;
  c[3] = 0u;
  philox4x32_10(c, k0, k1);
  normal_pair(c[0], c[1], &g1, &g2);
  if (lin == plin) {
    *re = sqrt(N) * g1;
    *im = 0.0;
  } else {
    *re = half * g1;
    *im = lin > plin ? -half * g2 : half * g2;
  }
}

void oracle_fourier_noise(int sx, int sy, int sz, unsigned long long seed, unsigned int step, unsigned int fid,
                          double* out) {
  const uint32_t k0 = (uint32_t)(seed & 0xFFFFFFFFull), k1 = (uint32_t)(seed >> 32);
#pragma omp parallel for schedule(static)
  for (int kz = 0; kz < sz; ++kz)
    for (int ky = 0; ky < sy; ++ky)
      for (int kx = 0; kx < sx; ++kx) {
        double re, im;
        if (2 * kx > sx) {
          /* Hermitian partner (sx - kx, -ky, -kz), conjugated */
          mode(sx, sy, sz, k0, k1, step, fid, sx - kx, (sy - ky) % sy, (sz - kz) % sz, &re, &im);
          im = -im;
        } else {
          mode(sx, sy, sz, k0, k1, step, fid, kx, ky, kz, &re, &im);
        }
        const size_t i = (((size_t)kz * sy + ky) * sx + kx) * 2;
        out[i] = re;
        out[i + 1] = im;
      }
}
