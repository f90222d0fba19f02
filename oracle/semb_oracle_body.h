/* Body of the oracle restatement, instantiated once per precision by semb_oracle.c
 * with REAL (float|double), SQRTR (sqrtf|sqrt) and SFX (function-name suffix).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a CPU restatement of the reference's OpenMP
 * semblance search (CMP/OpenMP/src/main.cpp:67-260, CRS/OpenMP/src/main.cpp:84-359)
 * written as plain C.  Every arithmetic expression keeps the reference's operand
 * order and types (float/double promotion of the literals included) so that, built
 * with -ffp-contract=off, it reproduces the reference bit for bit.  It is the
 * checker for the CUDA path and the CPU baseline of the benchmark; nothing in the
 * product links it.
 *
 * Inputs are the arrays su_gather::linearize produces (CRS/OpenMP/src/su_gather.cpp:
 * 94-127): an inclusive prefix count of traces per CDP, the samples of all traces
 * back to back, and the raw integer header fields gx, gy, sx, sy, scalco per trace.
 * Parameters are passed as the values the reference's parser produced: stof()
 * results for CMP, stod() results for CRS, both widened to double.
 *
 * cdp_list (optional, n_list entries) restricts the search to those CDPs; the
 * neighbour lists and geometry still come from the whole gather.  Rows of CDPs
 * not in the list are left as the caller initialised them.
 *
 * Divergence (documented): where the reference converts a NaN or out-of-int-range
 * traveltime with (int)t, which is undefined behaviour in C (x86 gives INT_MIN and
 * the window test then depends on signed overflow; AArch64 saturates), this
 * restatement counts the trace as out of range.  Such traveltimes need a negative
 * t0^2 + c*h (a negative -c0) or a window past 2^31 samples. */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)

/* (int)t with the reference's meaning for every t the reference handles; returns 0
 * and sets *bad when t is NaN or outside the int range. */
static inline int CAT(trunc_int, SFX)(REAL t, int* bad) {
  if (!(t > -2147483648.0 && t < 2147483647.0)) { *bad = 1; return 0; }
  return (int)t;
}

/* Gap between the largest and the second-largest of n semblances (checker output,
 * not part of the reference's computation). */
static inline double CAT(top2_gap, SFX)(const REAL* v, int n) {
  double b1 = -1e300, b2 = -1e300;
  for (int i = 0; i < n; i++) {
    const double x = (double)v[i];
    if (x > b1) { b2 = b1; b1 = x; }
    else if (x > b2) b2 = x;
  }
  return n > 1 ? b1 - b2 : 1e300;
}

/* CMP: CMP/OpenMP/src/main.cpp:88-241 (grid :119-122, half-offsets :125-136,
 * semblance :149-204, argmax :207-222, output values :253-255). */
int CAT(semb_oracle_cmp, SFX)(int ncdps, const int32_t* ntraces_by_cdp_id, int ns, int dt_us,
                              const float* samples, const int32_t* gxi, const int32_t* gyi,
                              const int32_t* sxi, const int32_t* syi, const int32_t* scalcoi,
                              double c0_parsed, double c1_parsed, int nc, double tau_parsed,
                              int32_t* ctr, REAL* str, REAL* stk, float* out_c,
                              REAL* sem_all, double* seconds, const int32_t* cdp_list, int n_list) {
  const REAL c0 = (REAL)(c0_parsed * FACTOR);
  const REAL c1 = (REAL)(c1_parsed * FACTOR);
  const REAL itau = (REAL)tau_parsed;
  if (ncdps <= 0 || nc <= 0 || ns <= 0) return -1;
  const int ttraces = ntraces_by_cdp_id[ncdps - 1];
  const REAL inc = (c1 - c0) * (1.0f / (REAL)nc);

  REAL* c = (REAL*)malloc(sizeof(REAL) * (size_t)nc);
  REAL* h = (REAL*)malloc(sizeof(REAL) * (size_t)(ttraces > 0 ? ttraces : 1));
  REAL* num = (REAL*)malloc(sizeof(REAL) * (size_t)ns * nc);
  REAL* stt = (REAL*)malloc(sizeof(REAL) * (size_t)ns * nc);
  if (!c || !h || !num || !stt) { free(c); free(h); free(num); free(stt); return -2; }

  REAL dt = (REAL)dt_us;
  dt = dt / 1000000.0f;
  REAL idt = 1.0f / dt;
  int tau = ((int)(itau * idt) > 0) ? ((int)(itau * idt)) : 0;
  REAL w = (2 * tau) + 1;
  if (w > MAX_W_CMP) { free(c); free(h); free(num); free(stt); return -3; }

  double t_beg = omp_get_wtime();
  for (int i = 0; i < nc; i++) c[i] = c0 + inc * i;

#pragma omp parallel for
  for (int i = 0; i < ttraces; i++) {
    REAL _s = (REAL)scalcoi[i];
    if (-EPSILON < _s && _s < EPSILON) _s = 1.0;
    else if (_s < 0) _s = 1.0f / _s;
    REAL hx = ((REAL)gxi[i] - (REAL)sxi[i]) * _s;
    REAL hy = ((REAL)gyi[i] - (REAL)syi[i]) * _s;
    h[i] = 0.25 * (hx * hx + hy * hy) / FACTOR;
  }

  const int n_todo = cdp_list ? n_list : ncdps;
  for (int q_id = 0; q_id < n_todo; q_id++) {
    const int cdp_id = cdp_list ? cdp_list[q_id] : q_id;
    const int t_id0 = cdp_id > 0 ? ntraces_by_cdp_id[cdp_id - 1] : 0;
    const int t_idf = ntraces_by_cdp_id[cdp_id];
    const float* cdpsmpl = samples + (size_t)t_id0 * ns;

    const int t0_lo = semb_oracle_t0_lo < ns ? semb_oracle_t0_lo : ns;
    const int t0_hi = semb_oracle_t0_hi < ns ? semb_oracle_t0_hi : ns;
#pragma omp parallel for schedule(static)
    for (int i = t0_lo * nc; i < t0_hi * nc; i++) {
      REAL _num[MAX_W_CMP], _ac_squared = 0, _ac_linear = 0, _den = 0, m = 0;
      int err = 0;
      int c_id = i % nc;
      int t0 = i / nc;
      REAL _c = c[c_id];
      REAL _t0 = dt * t0;
      _t0 = _t0 * _t0;
      for (int j = 0; j < w; j++) _num[j] = 0.0f;
      for (int t_id = t_id0; t_id < t_idf; t_id++) {
        REAL t = SQRTR(_t0 + _c * h[t_id]) * idt;
        int bad = 0;
        int it = CAT(trunc_int, SFX)(t, &bad);
        int ittau = it - tau;
        REAL x = t - (REAL)it;
        if (!bad && ittau >= 0 && it + tau + 1 < ns) {
          size_t k1 = (size_t)ittau + (size_t)(t_id - t_id0) * ns;
          REAL sk1p1 = cdpsmpl[k1], sk1;
          for (int j = 0; j < w; j++) {
            k1++;
            sk1 = sk1p1;
            sk1p1 = cdpsmpl[k1];
            REAL v = (sk1p1 - sk1) * x + sk1;
            _num[j] += v;
            _den += v * v;
            _ac_linear += v;
          }
          m++;
        } else {
          err++;
        }
      }
      for (int j = 0; j < w; j++) _ac_squared += _num[j] * _num[j];
      if (_den > EPSILON && m > EPSILON && w > EPSILON && err < 2) {
        num[i] = _ac_squared / (_den * m);
        stt[i] = _ac_linear / (w * m);
      } else {
        num[i] = -1.0f;
        stt[i] = -1.0f;
      }
    }

    if (sem_all) memcpy(sem_all + (size_t)cdp_id * ns * nc, num, sizeof(REAL) * (size_t)ns * nc);

#pragma omp parallel for
    for (int t0 = t0_lo; t0 < t0_hi; t0++) {
      REAL max_sem = 0.0f;
      int max_c = -1;
      for (int it = t0 * nc; it < (t0 + 1) * nc; it++) {
        if (num[it] > max_sem) { max_sem = num[it]; max_c = it; }
      }
      size_t o = (size_t)cdp_id * ns + t0;
      if (semb_oracle_top2) semb_oracle_top2[o] = CAT(top2_gap, SFX)(num + (size_t)t0 * nc, nc);
      ctr[o] = max_c % nc;
      str[o] = max_sem;
      stk[o] = max_c > -1 ? stt[max_c] : 0.0f;
    }
  }
  if (seconds) *seconds = omp_get_wtime() - t_beg;

  if (out_c) {
    for (size_t o = 0; o < (size_t)ncdps * ns; o++)
      out_c[o] = ctr[o] < 0 ? 0.0f : (c0 + inc * ctr[o]) / FACTOR;
  }
  free(c); free(h); free(num); free(stt);
  return 0;
}

/* CRS: CRS/OpenMP/src/main.cpp:85-359 (grid :155-160, geometry :163-177, aperture
 * :179-204 and :289-317, semblance :209-267, argmax :270-285, outputs :348-352).
 * nbr_off[ncdps+1] / nbr[] hold each CDP's neighbour list in ascending order
 * (su_gather.cpp:70-87). */
int CAT(semb_oracle_crs, SFX)(int ncdps, const int32_t* ntraces_by_cdp_id, int ns, int dt_us,
                              const float* samples, const int32_t* gxi, const int32_t* gyi,
                              const int32_t* sxi, const int32_t* syi, const int32_t* scalcoi,
                              const int32_t* nbr_off, const int32_t* nbr,
                              double a0_parsed, double a1_parsed, int na,
                              double b0_parsed, double b1_parsed, int nb,
                              double c0_parsed, double c1_parsed, int nc, double tau_parsed,
                              int32_t* ctr, REAL* str, REAL* stk,
                              float* out_a, float* out_b, float* out_c,
                              REAL* sem_all, double* seconds, int64_t* n_semblance_traces,
                              const int32_t* cdp_list, int n_list) {
  const REAL a0 = (REAL)a0_parsed, a1 = (REAL)a1_parsed;
  const REAL b0 = (REAL)b0_parsed, b1 = (REAL)b1_parsed;
  const REAL c0 = (REAL)(c0_parsed * FACTOR), c1 = (REAL)(c1_parsed * FACTOR);
  const REAL itau = (REAL)tau_parsed;
  if (ncdps <= 0 || na <= 0 || nb <= 0 || nc <= 0 || ns <= 0) return -1;
  const int ttraces = ntraces_by_cdp_id[ncdps - 1];
  const REAL inc_a = (a1 - a0) * (1.0 / (REAL)na);
  const REAL inc_b = (b1 - b0) * (1.0 / (REAL)nb);
  const REAL inc_c = (c1 - c0) * (1.0 / (REAL)nc);
  const int npar = na * nb * nc;

  int max_ap = 0;
  for (int i = 0; i < ncdps; i++) {
    int n = 0;
    for (int q = nbr_off[i]; q < nbr_off[i + 1]; q++) {
      int cdp = nbr[q];
      n += ntraces_by_cdp_id[cdp] - (cdp > 0 ? ntraces_by_cdp_id[cdp - 1] : 0);
    }
    if (n > max_ap) max_ap = n;
  }

  REAL* pa = (REAL*)malloc(sizeof(REAL) * (size_t)npar);
  REAL* pb = (REAL*)malloc(sizeof(REAL) * (size_t)npar);
  REAL* pc = (REAL*)malloc(sizeof(REAL) * (size_t)npar);
  REAL* h0 = (REAL*)malloc(sizeof(REAL) * (size_t)(ttraces > 0 ? ttraces : 1));
  REAL* m0x = (REAL*)malloc(sizeof(REAL) * (size_t)(ttraces > 0 ? ttraces : 1));
  REAL* m0y = (REAL*)malloc(sizeof(REAL) * (size_t)(ttraces > 0 ? ttraces : 1));
  REAL* num = (REAL*)malloc(sizeof(REAL) * (size_t)ns * npar);
  REAL* stt = (REAL*)malloc(sizeof(REAL) * (size_t)ns * npar);
  size_t apn = (size_t)(max_ap > 0 ? max_ap : 1);
  float* cdpsmpl = (float*)malloc(sizeof(float) * apn * ns);
  REAL* m2 = (REAL*)malloc(sizeof(REAL) * apn);
  REAL* m = (REAL*)malloc(sizeof(REAL) * apn);
  REAL* h = (REAL*)malloc(sizeof(REAL) * apn);
  if (!pa || !pb || !pc || !h0 || !m0x || !m0y || !num || !stt || !cdpsmpl || !m2 || !m || !h) {
    free(pa); free(pb); free(pc); free(h0); free(m0x); free(m0y); free(num); free(stt);
    free(cdpsmpl); free(m2); free(m); free(h);
    return -2;
  }

  REAL dt = (REAL)dt_us;
  dt = dt / 1000000.0f;
  REAL idt = 1.0f / dt;
  int tau = (int)(itau * idt) > 0 ? (int)(itau * idt) : 0;
  int w = (2 * tau) + 1;
  int rc = 0;
  if (w > MAX_W_CRS) rc = -3;
  int64_t nsem = 0;

  double t_beg = omp_get_wtime();
  for (int i = 0; rc == 0 && i < npar; i++) {
    pa[i] = a0 + inc_a * (i / (nc * nb));
    pb[i] = b0 + inc_b * ((i / nc) % nb);
    pc[i] = c0 + inc_c * (i % nc);
  }

#pragma omp parallel for
  for (int i = 0; i < ttraces; i++) {
    REAL _s = (REAL)scalcoi[i];
    if (-EPSILON < _s && _s < EPSILON) _s = 1.0;
    else if (_s < 0) _s = 1.0f / _s;
    m0x[i] = ((REAL)gxi[i] + (REAL)sxi[i]) * _s * 0.5;
    m0y[i] = ((REAL)gyi[i] + (REAL)syi[i]) * _s * 0.5;
    REAL hx = ((REAL)gxi[i] - (REAL)sxi[i]) * _s;
    REAL hy = ((REAL)gyi[i] - (REAL)syi[i]) * _s;
    h0[i] = 0.25 * (hx * hx + hy * hy) / FACTOR;
  }

  const int n_todo = cdp_list ? n_list : ncdps;
  for (int q_id = 0; rc == 0 && q_id < n_todo; q_id++) {
    const int cdp_id = cdp_list ? cdp_list[q_id] : q_id;
    const int first = cdp_id > 0 ? ntraces_by_cdp_id[cdp_id - 1] : 0;
    const REAL m0x_cdp_id = m0x[first], m0y_cdp_id = m0y[first];
    int size = 0;
    for (int q = nbr_off[cdp_id]; q < nbr_off[cdp_id + 1]; q++) {
      int cdp = nbr[q];
      int t_id0 = cdp > 0 ? ntraces_by_cdp_id[cdp - 1] : 0;
      int t_idf = ntraces_by_cdp_id[cdp];
      memcpy(cdpsmpl + (size_t)size * ns, samples + (size_t)t_id0 * ns, sizeof(float) * (size_t)(t_idf - t_id0) * ns);
      for (int it = 0; it < t_idf - t_id0; it++) {
        REAL dx = m0x[t_id0 + it] - m0x_cdp_id;
        REAL dy = m0y[t_id0 + it] - m0y_cdp_id;
        if (semb_oracle_dm_signed) {
          /* signed displacement along the azimuth (no reference counterpart) */
          const REAL md = dx * (REAL)semb_oracle_dm_cos + dy * (REAL)semb_oracle_dm_sin;
          m[size + it] = md;
          m2[size + it] = md * md;
        } else {
          REAL _m2 = dx * dx + dy * dy;
          m2[size + it] = _m2;
          m[size + it] = SQRTR(_m2);
        }
        h[size + it] = h0[t_id0 + it];
      }
      size += t_idf - t_id0;
    }
    nsem += size;

    const int t0_lo = semb_oracle_t0_lo < ns ? semb_oracle_t0_lo : ns;
    const int t0_hi = semb_oracle_t0_hi < ns ? semb_oracle_t0_hi : ns;
    /* a t0 range that skips t0 = 0 still evaluates that row: its candidate 0 gives
     * the stack of the t0 without a pick (stt[max_par] with max_par = 0 below) */
    const int extra = (t0_lo > 0 && t0_lo < t0_hi) ? 1 : 0;
    const int nrows = (t0_hi > t0_lo ? t0_hi - t0_lo : 0) + extra;
#pragma omp parallel for collapse(2) schedule(static)
    for (int row = 0; row < nrows; row++) {
      for (int par_id = 0; par_id < npar; par_id++) {
        const int t0 = extra ? (row == 0 ? 0 : t0_lo + row - 1) : t0_lo + row;
        REAL _num[MAX_W_CRS], _ac_squared = 0, _ac_linear = 0, _den = 0, mm = 0;
        int err = 0;
        int id = t0 * npar + par_id;
        REAL pA = pa[par_id], pB = pb[par_id], pC = pc[par_id];
        REAL _t0 = dt * t0;
        for (int j = 0; j < w; j++) _num[j] = 0.0f;
        for (int k = 0; k < size; k++) {
          REAL _m2 = m2[k];
          REAL t = _t0 + pA * m[k];
          t = t * t + pB * _m2 + pC * h[k];
          t = t < 0.0 ? -1 : SQRTR(t);
          int bad = 0;
          int it = CAT(trunc_int, SFX)(t * idt, &bad);
          int ittau = it - tau;
          REAL x = t * idt - (REAL)it;
          if (!bad && ittau >= 0 && it + tau + 1 < ns) {
            size_t k1 = (size_t)ittau + (size_t)k * ns;
            REAL sk1p1 = cdpsmpl[k1], sk1;
            for (int j = 0; j < w; j++) {
              k1++;
              sk1 = sk1p1;
              sk1p1 = cdpsmpl[k1];
              REAL v = (sk1p1 - sk1) * x + sk1;
              _num[j] += v;
              _den += v * v;
              _ac_linear += v;
            }
            mm++;
          } else {
            err++;
          }
        }
        for (int j = 0; j < w; j++) _ac_squared += _num[j] * _num[j];
        if (_den > EPSILON && mm > EPSILON && w > EPSILON && err < 2) {
          num[id] = _ac_squared / (_den * mm);
          stt[id] = _ac_linear / (w * mm);
        } else {
          num[id] = 0.0f;
          stt[id] = 0.0f;
        }
      }
    }

    if (sem_all) memcpy(sem_all + (size_t)cdp_id * ns * npar, num, sizeof(REAL) * (size_t)ns * npar);

#pragma omp parallel for
    for (int t0 = t0_lo; t0 < t0_hi; t0++) {
      REAL max_sem = 0.0f;
      int max_par = 0;
      for (int it = t0 * npar; it < (t0 + 1) * npar; it++) {
        if (num[it] > max_sem) { max_sem = num[it]; max_par = it; }
      }
      size_t o = (size_t)cdp_id * ns + t0;
      if (semb_oracle_top2) semb_oracle_top2[o] = CAT(top2_gap, SFX)(num + (size_t)t0 * npar, npar);
      ctr[o] = max_par % npar;
      str[o] = max_sem;
      stk[o] = stt[max_par];
    }
  }
  if (seconds) *seconds = omp_get_wtime() - t_beg;
  if (n_semblance_traces) *n_semblance_traces = nsem;

  if (rc == 0) {
    for (size_t o = 0; o < (size_t)ncdps * ns; o++) {
      if (out_a) out_a[o] = (a0 + inc_a * (ctr[o] / (nc * nb)));
      if (out_b) out_b[o] = (b0 + inc_b * ((ctr[o] / nc) % nb));
      if (out_c) out_c[o] = (c0 + inc_c * (ctr[o] % nc)) / FACTOR;
    }
  }
  free(pa); free(pb); free(pc); free(h0); free(m0x); free(m0y); free(num); free(stt);
  free(cdpsmpl); free(m2); free(m); free(h);
  return rc;
}

/* CRS-DE: differential-evolution search over (A, B, C), the method of the
 * reference's crs-ocl-de (README.md:86-106, flags of crs-ocl-de plus -ngen), whose
 * source is not in the reference.  This restates the library's definition of it
 * (no reference code to follow):
 *   population  NP = na * nb * nc individuals, started on the search grid (the
 *               exhaustive search's candidates, in its index order);
 *   generation  DE/rand/1/bin for every individual i against the population of
 *               the previous generation: r1, r2, r3 distinct and != i, jrand in
 *               0..2, trial_d = x_r1,d + F * (x_r2,d - x_r3,d) where u_d < CR or
 *               d == jrand, else x_i,d; clamped to [lo_d, hi_d] = [a0, a1],
 *               [b0, b1], [c0, c1] (C in 1e6-scaled units); F = 0.5, CR = 0.9;
 *               the trial replaces i when its semblance is >= i's;
 *   random      counter-based: de_key(cdp, t0, gen, i, slot) (splitmix64 chain),
 *               integers by modulo, u_d = (key >> 40) * 2^-24;
 *   pick        the individual with the largest semblance (lowest index on ties);
 *               none positive: the first grid candidate and the stack of item
 *               (t0 = 0, candidate 0), as the grid search reports.
 * The semblance of one (t0, A, B, C) is the CRS operator of main.cpp:209-267.
 * Outputs a, b, c (C divided back by 1e6), str, stk per (CDP, t0). */
#ifndef SEMB_DE_HELPERS
#define SEMB_DE_HELPERS
static inline uint64_t semb_de_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline uint64_t semb_de_key(int cdp, int t0, int gen, int i, int slot) {
  uint64_t z = semb_de_mix(((uint64_t)(uint32_t)cdp << 32) | (uint32_t)t0);
  z = semb_de_mix(z ^ (((uint64_t)(uint32_t)gen << 32) | (uint32_t)i));
  return semb_de_mix(z ^ (uint64_t)(uint32_t)slot);
}
/* r1, r2, r3: distinct, all != i (requires np >= 4) */
static inline void semb_de_pick3(int cdp, int t0, int gen, int i, int np, int* r) {
  int ex[4];
  int nex = 1;
  ex[0] = i;
  for (int q = 0; q < 3; ++q) {
    int v = (int)(semb_de_key(cdp, t0, gen, i, q) % (uint64_t)(np - nex));
    /* the v-th index not excluded: step past the excluded ones in ascending order */
    int sorted[4];
    for (int a = 0; a < nex; ++a) sorted[a] = ex[a];
    for (int a = 1; a < nex; ++a)
      for (int b = a; b > 0 && sorted[b - 1] > sorted[b]; --b) {
        int tmp = sorted[b]; sorted[b] = sorted[b - 1]; sorted[b - 1] = tmp;
      }
    for (int a = 0; a < nex; ++a)
      if (v >= sorted[a]) ++v;
    r[q] = v;
    ex[nex++] = v;
  }
}
#endif

/* semblance and stack of one (t0, A, B, C) on an assembled aperture */
static inline void CAT(crs_eval_one, SFX)(REAL pA, REAL pB, REAL pC, int t0, REAL dt, REAL idt, int tau, int w,
                                          int ns, int size, const float* cdpsmpl, const REAL* m, const REAL* m2,
                                          const REAL* h, REAL* sem, REAL* stk) {
  REAL _num[MAX_W_CRS], _ac_squared = 0, _ac_linear = 0, _den = 0, mm = 0;
  int err = 0;
  REAL _t0 = dt * t0;
  for (int j = 0; j < w; j++) _num[j] = 0.0f;
  for (int k = 0; k < size; k++) {
    REAL _m2 = m2[k];
    REAL t = _t0 + pA * m[k];
    t = t * t + pB * _m2 + pC * h[k];
    t = t < 0.0 ? -1 : SQRTR(t);
    int bad = 0;
    int it = CAT(trunc_int, SFX)(t * idt, &bad);
    int ittau = it - tau;
    REAL x = t * idt - (REAL)it;
    if (!bad && ittau >= 0 && it + tau + 1 < ns) {
      size_t k1 = (size_t)ittau + (size_t)k * ns;
      REAL sk1p1 = cdpsmpl[k1], sk1;
      for (int j = 0; j < w; j++) {
        k1++;
        sk1 = sk1p1;
        sk1p1 = cdpsmpl[k1];
        REAL v = (sk1p1 - sk1) * x + sk1;
        _num[j] += v;
        _den += v * v;
        _ac_linear += v;
      }
      mm++;
    } else {
      err++;
    }
  }
  for (int j = 0; j < w; j++) _ac_squared += _num[j] * _num[j];
  if (_den > EPSILON && mm > EPSILON && w > EPSILON && err < 2) {
    *sem = _ac_squared / (_den * mm);
    *stk = _ac_linear / (w * mm);
  } else {
    *sem = 0.0f;
    *stk = 0.0f;
  }
}

int CAT(semb_oracle_crs_de, SFX)(int ncdps, const int32_t* ntraces_by_cdp_id, int ns, int dt_us,
                                 const float* samples, const int32_t* gxi, const int32_t* gyi,
                                 const int32_t* sxi, const int32_t* syi, const int32_t* scalcoi,
                                 const int32_t* nbr_off, const int32_t* nbr,
                                 double a0_parsed, double a1_parsed, int na,
                                 double b0_parsed, double b1_parsed, int nb,
                                 double c0_parsed, double c1_parsed, int nc, double tau_parsed, int ngen,
                                 float* out_a, float* out_b, float* out_c, REAL* str, REAL* stk,
                                 const int32_t* cdp_list, int n_list) {
  const REAL a0 = (REAL)a0_parsed, a1 = (REAL)a1_parsed;
  const REAL b0 = (REAL)b0_parsed, b1 = (REAL)b1_parsed;
  const REAL c0 = (REAL)(c0_parsed * FACTOR), c1 = (REAL)(c1_parsed * FACTOR);
  const REAL itau = (REAL)tau_parsed;
  if (ncdps <= 0 || na <= 0 || nb <= 0 || nc <= 0 || ns <= 0 || ngen < 0) return -1;
  const int ttraces = ntraces_by_cdp_id[ncdps - 1];
  const REAL inc_a = (a1 - a0) * (1.0 / (REAL)na);
  const REAL inc_b = (b1 - b0) * (1.0 / (REAL)nb);
  const REAL inc_c = (c1 - c0) * (1.0 / (REAL)nc);
  const int np = na * nb * nc;
  const REAL lo[3] = {a0, b0, c0}, hi[3] = {a1, b1, c1};
  const REAL F = 0.5f, CR = 0.9f;

  int max_ap = 0;
  for (int i = 0; i < ncdps; i++) {
    int n = 0;
    for (int q = nbr_off[i]; q < nbr_off[i + 1]; q++) {
      int cdp = nbr[q];
      n += ntraces_by_cdp_id[cdp] - (cdp > 0 ? ntraces_by_cdp_id[cdp - 1] : 0);
    }
    if (n > max_ap) max_ap = n;
  }
  REAL* grid = (REAL*)malloc(sizeof(REAL) * 3 * (size_t)np);
  REAL* h0 = (REAL*)malloc(sizeof(REAL) * (size_t)(ttraces > 0 ? ttraces : 1));
  REAL* m0x = (REAL*)malloc(sizeof(REAL) * (size_t)(ttraces > 0 ? ttraces : 1));
  REAL* m0y = (REAL*)malloc(sizeof(REAL) * (size_t)(ttraces > 0 ? ttraces : 1));
  size_t apn = (size_t)(max_ap > 0 ? max_ap : 1);
  float* cdpsmpl = (float*)malloc(sizeof(float) * apn * ns);
  REAL* m2 = (REAL*)malloc(sizeof(REAL) * apn);
  REAL* m = (REAL*)malloc(sizeof(REAL) * apn);
  REAL* h = (REAL*)malloc(sizeof(REAL) * apn);
  if (!grid || !h0 || !m0x || !m0y || !cdpsmpl || !m2 || !m || !h) {
    free(grid); free(h0); free(m0x); free(m0y); free(cdpsmpl); free(m2); free(m); free(h);
    return -2;
  }
  REAL dt = (REAL)dt_us;
  dt = dt / 1000000.0f;
  REAL idt = 1.0f / dt;
  int tau = (int)(itau * idt) > 0 ? (int)(itau * idt) : 0;
  int w = (2 * tau) + 1;
  if (w > MAX_W_CRS) {
    free(grid); free(h0); free(m0x); free(m0y); free(cdpsmpl); free(m2); free(m); free(h);
    return -3;
  }
  for (int i = 0; i < np; i++) {
    grid[3 * i] = a0 + inc_a * (i / (nc * nb));
    grid[3 * i + 1] = b0 + inc_b * ((i / nc) % nb);
    grid[3 * i + 2] = c0 + inc_c * (i % nc);
  }
  for (int i = 0; i < ttraces; i++) {
    REAL _s = (REAL)scalcoi[i];
    if (-EPSILON < _s && _s < EPSILON) _s = 1.0;
    else if (_s < 0) _s = 1.0f / _s;
    m0x[i] = ((REAL)gxi[i] + (REAL)sxi[i]) * _s * 0.5;
    m0y[i] = ((REAL)gyi[i] + (REAL)syi[i]) * _s * 0.5;
    REAL hx = ((REAL)gxi[i] - (REAL)sxi[i]) * _s;
    REAL hy = ((REAL)gyi[i] - (REAL)syi[i]) * _s;
    h0[i] = 0.25 * (hx * hx + hy * hy) / FACTOR;
  }
  const int n_todo = cdp_list ? n_list : ncdps;
  for (int q_id = 0; q_id < n_todo; q_id++) {
    const int cdp_id = cdp_list ? cdp_list[q_id] : q_id;
    const int first = cdp_id > 0 ? ntraces_by_cdp_id[cdp_id - 1] : 0;
    const REAL m0x_cdp_id = m0x[first], m0y_cdp_id = m0y[first];
    int size = 0;
    for (int q = nbr_off[cdp_id]; q < nbr_off[cdp_id + 1]; q++) {
      int cdp = nbr[q];
      int t_id0 = cdp > 0 ? ntraces_by_cdp_id[cdp - 1] : 0;
      int t_idf = ntraces_by_cdp_id[cdp];
      memcpy(cdpsmpl + (size_t)size * ns, samples + (size_t)t_id0 * ns, sizeof(float) * (size_t)(t_idf - t_id0) * ns);
      for (int it = 0; it < t_idf - t_id0; it++) {
        REAL dx = m0x[t_id0 + it] - m0x_cdp_id;
        REAL dy = m0y[t_id0 + it] - m0y_cdp_id;
        if (semb_oracle_dm_signed) {
          const REAL md = dx * (REAL)semb_oracle_dm_cos + dy * (REAL)semb_oracle_dm_sin;
          m[size + it] = md;
          m2[size + it] = md * md;
        } else {
          REAL _m2 = dx * dx + dy * dy;
          m2[size + it] = _m2;
          m[size + it] = SQRTR(_m2);
        }
        h[size + it] = h0[t_id0 + it];
      }
      size += t_idf - t_id0;
    }
    /* stack of item (t0 = 0, candidate 0), reported where nothing is picked */
    REAL sem00, stk00;
    CAT(crs_eval_one, SFX)(grid[0], grid[1], grid[2], 0, dt, idt, tau, w, ns, size, cdpsmpl, m, m2, h, &sem00,
                           &stk00);
#pragma omp parallel for schedule(dynamic, 4)
    for (int t0 = 0; t0 < ns; t0++) {
      REAL* pop = (REAL*)malloc(sizeof(REAL) * 5 * (size_t)np);   /* a, b, c, sem, stk */
      REAL* tri = (REAL*)malloc(sizeof(REAL) * 5 * (size_t)np);
      if (!pop || !tri) { free(pop); free(tri); continue; }
      for (int i = 0; i < np; i++) {
        pop[5 * i] = grid[3 * i];
        pop[5 * i + 1] = grid[3 * i + 1];
        pop[5 * i + 2] = grid[3 * i + 2];
        CAT(crs_eval_one, SFX)(pop[5 * i], pop[5 * i + 1], pop[5 * i + 2], t0, dt, idt, tau, w, ns, size, cdpsmpl,
                               m, m2, h, &pop[5 * i + 3], &pop[5 * i + 4]);
      }
      for (int gen = 1; np >= 4 && gen <= ngen; gen++) {
        for (int i = 0; i < np; i++) {
          int r[3];
          semb_de_pick3(cdp_id, t0, gen, i, np, r);
          const int jrand = (int)(semb_de_key(cdp_id, t0, gen, i, 3) % 3u);
          for (int d = 0; d < 3; d++) {
            const float u = (float)(semb_de_key(cdp_id, t0, gen, i, 4 + d) >> 40) * (1.0f / 16777216.0f);
            REAL v = pop[5 * i + d];
            if (u < (float)CR || d == jrand) {
              const REAL diff = pop[5 * r[1] + d] - pop[5 * r[2] + d];
              const REAL step = F * diff;
              v = pop[5 * r[0] + d] + step;
            }
            v = v < lo[d] ? lo[d] : (v > hi[d] ? hi[d] : v);
            tri[5 * i + d] = v;
          }
          CAT(crs_eval_one, SFX)(tri[5 * i], tri[5 * i + 1], tri[5 * i + 2], t0, dt, idt, tau, w, ns, size,
                                 cdpsmpl, m, m2, h, &tri[5 * i + 3], &tri[5 * i + 4]);
        }
        for (int i = 0; i < np; i++)
          if (tri[5 * i + 3] >= pop[5 * i + 3])
            for (int d = 0; d < 5; d++) pop[5 * i + d] = tri[5 * i + d];
      }
      int best = -1;
      REAL bs = 0.0f;
      for (int i = 0; i < np; i++)
        if (pop[5 * i + 3] > bs) { bs = pop[5 * i + 3]; best = i; }
      const size_t o = (size_t)cdp_id * ns + t0;
      if (best < 0) {
        out_a[o] = (float)grid[0];
        out_b[o] = (float)grid[1];
        out_c[o] = (float)(grid[2] / FACTOR);
        str[o] = 0.0f;
        stk[o] = stk00;
      } else {
        out_a[o] = (float)pop[5 * best];
        out_b[o] = (float)pop[5 * best + 1];
        out_c[o] = (float)(pop[5 * best + 2] / FACTOR);
        str[o] = bs;
        stk[o] = pop[5 * best + 4];
      }
      free(pop);
      free(tri);
    }
  }
  free(grid); free(h0); free(m0x); free(m0y); free(cdpsmpl); free(m2); free(m); free(h);
  return 0;
}

#undef CAT
#undef CAT_
