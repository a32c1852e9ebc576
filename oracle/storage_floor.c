/* storage_floor.c -- TEST / MEASUREMENT INFRASTRUCTURE, not product code.
 *
 * The rounding floor of each candidate storage of the D3Q19 populations,
 * measured on the CPU: a two-array restatement of the sphere-channel step
 * (BGK relaxation as src/lbm/solver.cpp:601-604 performs it, here on the
 * scaled deviation v = S (f - w) / w of the dense-box engine; halfway
 * bounce-back on the sphere; equilibrium inlet at x = 0; zero-gradient outlet
 * at x = nx - 1; free slip on the y and z faces) in which every population is
 * rounded to the candidate storage after each collision.  Run against the
 * same step in FP64 (store 0), the velocity error isolates what the storage
 * format costs.  The GPU engine itself is measured by bench.py's accuracy
 * workload; this program answers which 16-bit formats are worth building.
 *
 * usage: storage_floor nx ny nz R cx cy cz tau steps store arith out.bin
 *   store: 0 FP64; 1 FP32 of the shifted state s = v - S P(U);
 *          2 FP16 of v (no shift); 4 FP16 of s;
 *          14 FP16 of s with stochastic rounding (a hashed random offset
 *             below the FP16 ulp, then rounding toward zero);
 *          6 a 16-bit float of 1 sign, 4 exponent and 11 mantissa bits
 *            (Lehmann et al., Phys. Rev. E 106, 015308 (2022)) of s / S x 4:
 *            12 significant bits, normal range [2^-14, 2), saturating;
 *          7 a 16-bit float of 1 sign, 3 exponent and 12 mantissa bits of
            s / S x 4: 13 significant bits, normal range [2^-6, 2),
            subnormal below, saturating;
          8 16-bit fixed point of s: round(s / S x 2^15) / 2^15, saturating;
          9 block floating point of s: per cell, 16-bit integers times one
            power-of-two scale 2^(e - 15) with 2^e >= the cell's max |s|;
          10 the same with the scale of the slot's owner, as the AA pattern
            would hold it: set by the owner when it rewrites its own slots
            (even steps, one bit of headroom), used by the values its
            neighbours push into its slots (odd steps), saturating
 *   arith: 0 FP64 on v; 2 FP32 on the shifted state (the engine's
 *          single-precision collision in the same operation order)
 * out.bin: rho, ux, uy, uz per cell (FP64), x fastest.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static const int C[19][3] = {{-1, 0, 0}, {1, 0, 0},  {0, -1, 0},  {0, 1, 0},  {0, 0, -1},  {0, 0, 1},  {-1, -1, 0},
                             {-1, 1, 0}, {1, -1, 0}, {1, 1, 0},   {-1, 0, -1}, {-1, 0, 1}, {1, 0, -1}, {1, 0, 1},
                             {0, -1, -1}, {0, -1, 1}, {0, 1, -1}, {0, 1, 1},  {0, 0, 0}};
static const int OPP[19] = {1, 0, 3, 2, 5, 4, 9, 8, 7, 6, 13, 12, 11, 10, 17, 16, 15, 14, 18};
static double    W[19], K[19];
static int       smode;

static uint32_t hash3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u ^ c * 0xC2B2AE3Du;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  h ^= h >> 12;
  h *= 0x297A2D39u;
  h ^= h >> 15;
  return h;
}

/* round to p significant bits, exponents below emin subnormal, saturating at maxv */
static double round_fp(double x, int p, int emin, double maxv) {
  if(x == 0) return 0;
  const double a = fabs(x);
  if(a >= maxv) return copysign(maxv, x);
  int e;
  frexp(a, &e);
  int lead = e - 1;
  if(lead < emin) lead = emin;
  const double q = ldexp(1.0, lead - (p - 1));
  return copysign(nearbyint(a / q) * q, x);
}

/* store 9: the cell's 19 values as 16-bit integers with one power-of-two
   scale per cell (a shared exponent: block floating point), 2^e >= max |x| */
static void store_block(double* x) {
  double m = 0;
  for(int q = 0; q < 19; ++q) m = fmax(m, fabs(x[q]));
  if(m == 0) return;
  int e;
  frexp(m, &e);
  const double sc = ldexp(1.0, e - 15);
  for(int q = 0; q < 19; ++q) {
    double v = nearbyint(x[q] / sc);
    if(v > 32767) v = 32767;
    if(v < -32767) v = -32767;
    x[q] = v * sc;
  }
}

/* store 10: the same integers with the scale of the slot's owner cell: a cell
   sets its exponent when it rewrites all its own slots (the even AA step,
   from its post-collision values, `headroom` bits above their maximum), and
   values pushed into its slots in the odd step use it, saturating */
static void round_with(double* x, int e) {
  const double sc = ldexp(1.0, e - 15);
  for(int q = 0; q < 19; ++q) {
    double v = nearbyint(x[q] / sc);
    if(v > 32767) v = 32767;
    if(v < -32767) v = -32767;
    x[q] = v * sc;
  }
}
static int store_owner(double* x, int headroom, double also) {
  double m = also;
  for(int q = 0; q < 19; ++q) m = fmax(m, fabs(x[q]));
  int e = -10; /* a floor: a cell at the free stream (all values ~0) still takes what its neighbours push */
  if(m > 0) {
    int em;
    frexp(m, &em);
    if(em > e) e = em;
  }
  e += headroom;
  round_with(x, e);
  return e;
}

/* the stored value of x (state units: v or s) of direction q, cell i, step t */
static double store(double x, int q, uint32_t i, uint32_t t) {
  switch(smode) {
    case 0: return x;
    case 1: return (float)x;
    case 2:
    case 4: return round_fp(x, 11, -14, 65504.0);
    case 14: {
      const double a = fabs(x);
      if(a == 0) return 0;
      int e;
      frexp(a, &e);
      int lead = e - 1;
      if(lead < -14) lead = -14;
      const double ulp = ldexp(1.0, lead - 10);
      const double r   = (hash3(i, (uint32_t)q, t) & 0xFFFFu) / 65536.0;
      return copysign(floor(a / ulp + r) * ulp, x);
    }
    case 6: return round_fp(x / 4096.0 * 4.0, 12, -14, 2.0 - ldexp(1, -11)) / 4.0 * 4096.0;
    case 7: return round_fp(x / 4096.0 * 4.0, 13, -6, 2.0 - ldexp(1, -12)) / 4.0 * 4096.0;
    case 8: {
      double v = nearbyint(x / 4096.0 * 32768.0);
      if(v > 32767) v = 32767;
      if(v < -32768) v = -32768;
      return v / 32768.0 * 4096.0;
    }
  }
  return x;
}

int main(int argc, char** argv) {
  if(argc < 13) {
    fprintf(stderr, "usage: %s nx ny nz R cx cy cz tau steps store arith out.bin\n", argv[0]);
    return 2;
  }
  const int    nx = atoi(argv[1]), ny = atoi(argv[2]), nz = atoi(argv[3]);
  const double R = atof(argv[4]), cx = atof(argv[5]), cy = atof(argv[6]), cz = atof(argv[7]), tau = atof(argv[8]);
  const long   steps = atol(argv[9]);
  smode              = atoi(argv[10]);
  const int   farith = atoi(argv[11]);
  const char* out    = argv[12];
  const double om = 1.0 / tau, u0 = 0.05, S = 4096.0;
  const int    shifted = smode != 0 && smode != 2;
  if(smode == 10 && steps % 2) fprintf(stderr, "store 10: an even number of steps ends on a full rewrite\n");
  const double U       = shifted ? u0 : 0.0;
  for(int q = 0; q < 19; ++q) {
    const int n2 = C[q][0] * C[q][0] + C[q][1] * C[q][1] + C[q][2] * C[q][2];
    W[q]         = n2 == 0 ? 1.0 / 3 : (n2 == 1 ? 1.0 / 18 : 1.0 / 36);
    const double cu = C[q][0] * U;
    K[q]            = S * (3 * cu + 4.5 * cu * cu - 1.5 * U * U);  /* the shift S P_q(U) */
  }
  const int64_t N  = (int64_t)nx * ny * nz;
  uint8_t*      fl = calloc(N, 1); /* 0 fluid, 1 solid, 2 inlet, 3 outlet */
  for(int z = 0; z < nz; ++z)
    for(int y = 0; y < ny; ++y)
      for(int x = 0; x < nx; ++x) {
        const int64_t i  = x + (int64_t)nx * (y + (int64_t)ny * z);
        const double  dx = x + 0.5 - cx, dy = y + 0.5 - cy, dz = z + 0.5 - cz;
        if(dx * dx + dy * dy + dz * dz < R * R) fl[i] = 1;
        if(x == 0) fl[i] = 2;
        if(x == nx - 1) fl[i] = 3;
      }
  /* pull table: slot of the post-collision value that streams into (k, i);
     a bounce is encoded negative (it changes the shift) */
  int64_t* src = malloc(sizeof(int64_t) * 19 * N);
  for(int z = 0; z < nz; ++z)
    for(int y = 0; y < ny; ++y)
      for(int x = 0; x < nx; ++x) {
        const int64_t i = x + (int64_t)nx * (y + (int64_t)ny * z);
        for(int k = 0; k < 19; ++k) {
          int px = x, py = y, pz = z;
          if(fl[i] == 3 && C[k][0] < 0) px = x - 1; /* zero-gradient outlet: the upstream cell's links */
          int c[3] = {C[k][0], C[k][1], C[k][2]}, s[3] = {px - c[0], py - c[1], pz - c[2]}, n[3] = {nx, ny, nz}, p[3] = {px, py, pz};
          int bb = 0;
          for(int a = 0; a < 3; ++a)
            if(s[a] < 0 || s[a] >= n[a]) {
              if(a == 0) bb = 1;
              else {
                s[a] = p[a];
                c[a] = -c[a]; /* free slip: the mirrored direction of the same cell */
              }
            }
          const int64_t own = px + (int64_t)nx * (py + (int64_t)ny * pz), sc = s[0] + (int64_t)nx * (s[1] + (int64_t)ny * s[2]);
          int           q   = -1;
          for(int m = 0; m < 19; ++m)
            if(C[m][0] == c[0] && C[m][1] == c[1] && C[m][2] == c[2]) q = m;
          if(bb || fl[sc] == 1) src[k * N + i] = -(OPP[k] * N + own) - 1;
          else src[k * N + i] = q * N + sc;
        }
      }
  double* f  = malloc(sizeof(double) * 19 * N);
  double* fs = malloc(sizeof(double) * 19 * N);
  int*    ex = calloc(N, sizeof(int)); /* store 10: the slot owner's exponent */
  double  feq0[19];
  for(int q = 0; q < 19; ++q) {
    const double cu = C[q][0] * u0;
    feq0[q]         = S * (3 * cu + 4.5 * cu * cu - 1.5 * u0 * u0) - K[q];
    if(smode != 9) feq0[q] = store(feq0[q], q, 0, 0);
  }
  if(smode == 9) store_block(feq0);
  for(int q = 0; q < 19; ++q)
    for(int64_t i = 0; i < N; ++i) f[q * N + i] = fl[i] == 1 ? 0 : feq0[q];
  for(long t = 0; t < steps; ++t) {
#pragma omp parallel for schedule(static)
    for(int64_t i = 0; i < N; ++i) {
      if(fl[i] == 1) continue;
      if(fl[i] == 2) {
        for(int q = 0; q < 19; ++q) fs[q * N + i] = feq0[q];
        continue;
      }
      double o[19];
      if(farith == 2) {
        const float Sf = 4096.f, IS = 1.f / 4096.f, omf = (float)om, Uf = (float)U;
        float       sv[19], r0 = 0, j[3] = {0, 0, 0};
        for(int q = 0; q < 19; ++q) {
          sv[q]         = (float)f[q * N + i];
          const float w = (float)W[q];
          r0            = fmaf(w, sv[q], r0);
          for(int d = 0; d < 3; ++d) {
            if(C[q][d] > 0) j[d] = fmaf(w, sv[q], j[d]);
            if(C[q][d] < 0) j[d] = fmaf(-w, sv[q], j[d]);
          }
        }
        const float r = r0 * IS, rho = 1.f + r, irho = 1.f / rho;
        const float du[3] = {fmaf(-r, Uf, j[0] * IS) * irho, j[1] * IS * irho, j[2] * IS * irho};
        float       dusq  = du[0] * fmaf(2.f, Uf, du[0]);
        dusq              = fmaf(du[1], du[1], dusq);
        dusq              = fmaf(du[2], du[2], dusq);
        const float keep = 1.f - omf, oS = omf * Sf, A = oS * 4.5f * rho, B = oS * 3.f * rho;
        const float E0  = oS * fmaf(r, fmaf(-1.5f * Uf, Uf, 1.f), -1.5f * rho * dusq);
        const float E0x = fmaf(oS * 4.5f * r * Uf, Uf, E0), Bu = oS * 3.f * r * Uf;
        for(int q = 0; q < 19; ++q) {
          const int   cxq = C[q][0];
          const float cdu = C[q][0] * du[0] + C[q][1] * du[1] + C[q][2] * du[2];
          float       E, O;
          if(q == 18) {
            E = E0;
            O = 0;
          } else if(cxq == 0) {
            E = fmaf(A * cdu, cdu, E0);
            O = B * cdu;
          } else {
            E = fmaf(A * cdu, cdu + (cxq > 0 ? 2.f * Uf : -2.f * Uf), E0x);
            O = fmaf(B, cdu, cxq > 0 ? Bu : -Bu);
          }
          o[q] = fmaf(keep, sv[q], E + O);
        }
      } else {
        double v[19], r0 = 0, j[3] = {0, 0, 0};
        for(int q = 0; q < 19; ++q) {
          v[q] = (f[q * N + i] + K[q]) / S;
          r0 += W[q] * v[q];
          for(int d = 0; d < 3; ++d) j[d] += C[q][d] * W[q] * v[q];
        }
        const double rho = 1 + r0, u[3] = {j[0] / rho, j[1] / rho, j[2] / rho}, usq = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
        for(int q = 0; q < 19; ++q) {
          const double cu  = C[q][0] * u[0] + C[q][1] * u[1] + C[q][2] * u[2];
          const double veq = r0 + rho * (3 * cu + 4.5 * cu * cu - 1.5 * usq);
          o[q]             = S * (v[q] + om * (veq - v[q])) - K[q];
        }
      }
      if(smode == 9) store_block(o);
      if(smode == 10 && (t & 1) == 0) {
        /* even step: the cell rewrites its own slots; its exponent must also
           hold what a bounce will put there (its own population of the
           opposite direction plus the change of shift) */
        double bmax = 0;
        for(int k = 0; k < 19; ++k)
          if(src[k * N + i] < 0) bmax = fmax(bmax, fabs(o[OPP[k]] + K[OPP[k]] - K[k]));
        ex[i] = store_owner(o, 1, bmax);
      }
      for(int q = 0; q < 19; ++q)
        fs[q * N + i] = (smode == 9 || smode == 10) ? o[q] : store(o[q], q, (uint32_t)i, (uint32_t)t);
    }
#pragma omp parallel for schedule(static)
    for(int64_t i = 0; i < N; ++i) {
      if(fl[i] == 1) continue;
      if(fl[i] == 2) {
        for(int q = 0; q < 19; ++q) f[q * N + i] = feq0[q];
        continue;
      }
      for(int k = 0; k < 19; ++k) {
        const int64_t sidx = src[k * N + i];
        if(sidx >= 0) f[k * N + i] = fs[sidx];
        else f[k * N + i] = fs[-sidx - 1] + K[OPP[k]] - K[k]; /* bounced: the change of shift, added unrounded */
      }
      /* odd step: the values pushed into this cell's slots take its exponent
         from the last even step (saturating where they exceed it) */
      if(smode == 10 && (t & 1) == 1) {
        double v[19];
        for(int k = 0; k < 19; ++k) v[k] = f[k * N + i];
        round_with(v, ex[i]);
        for(int k = 0; k < 19; ++k) f[k * N + i] = v[k];
      }
    }
  }
  double* uo = malloc(sizeof(double) * 4 * N);
  for(int64_t i = 0; i < N; ++i) {
    double r0 = 0, j[3] = {0, 0, 0};
    for(int q = 0; q < 19; ++q) {
      const double v = (f[q * N + i] + K[q]) / S;
      r0 += W[q] * v;
      for(int d = 0; d < 3; ++d) j[d] += C[q][d] * W[q] * v;
    }
    const double rho = 1 + r0;
    uo[4 * i]        = fl[i] == 1 ? 0 : rho;
    for(int d = 0; d < 3; ++d) uo[4 * i + 1 + d] = fl[i] == 1 ? 0 : j[d] / rho;
  }
  FILE* fo = fopen(out, "wb");
  if(!fo) return 1;
  fwrite(uo, sizeof(double), 4 * N, fo);
  fclose(fo);
  free(uo);
  free(f);
  free(fs);
  free(src);
  free(fl);
  return 0;
}
