/*
 * CPU oracle for the minkasi pointing projections.  TEST INFRASTRUCTURE ONLY:
 * this file is compiled into oracle/mk_oracle.so and is called by tests/,
 * __graft_entry__.smoke() and the cpu_baseline / reference legs of bench.py,
 * always as the checker or the timed CPU baseline, never as the product path.
 *
 * It restates the arithmetic of the reference C library:
 *   orc_map2tod        <- map2tod_omp     minkasi/lib/minkasi.c:131-144
 *   orc_map2tod_serial <- map2tod_simple  minkasi/lib/minkasi.c:116-127
 *   orc_tod2map        <- tod2map_omp     minkasi/lib/minkasi.c:97-112
 *   orc_tod2map_serial <- tod2map_simple  minkasi/lib/minkasi.c:50-55
 *   orc_tod2map_atomic <- tod2map_atomic  minkasi/lib/minkasi.c:59-66
 * Layout as in the reference: dat is C-contiguous (ndet, ndata), the map is
 * flattened x*ny+y, ipix is int32 of the same shape as dat.
 *
 * Differences that do not change results beyond rounding order:
 *  - orc_tod2map reduces the per-thread private maps in thread-index order,
 *    so it is deterministic for a fixed thread count (the reference uses an
 *    omp critical section, i.e. arrival order);
 *  - an FP32 twin of each routine exists for the mixed-precision path;
 *  - sizes are 64-bit (the reference computes ndet*ndata in int).
 */
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_THREADS(nt) ((nt) > 0 ? (nt) : omp_get_max_threads())

/* ---- map2tod: dat[i] (+)= map[ipix[i]] ---------------------------------- */

void orc_map2tod(double *dat, const double *map, int64_t ndet, int64_t ndata,
                 const int32_t *ipix, int do_add, int nthread) {
  int64_t nn = ndet * ndata;
  if (do_add) {
#pragma omp parallel for num_threads(ORC_THREADS(nthread)) schedule(static)
    for (int64_t i = 0; i < nn; i++) dat[i] += map[ipix[i]];
  } else {
#pragma omp parallel for num_threads(ORC_THREADS(nthread)) schedule(static)
    for (int64_t i = 0; i < nn; i++) dat[i] = map[ipix[i]];
  }
}

void orc_map2tod_f32(float *dat, const float *map, int64_t ndet, int64_t ndata,
                     const int32_t *ipix, int do_add, int nthread) {
  int64_t nn = ndet * ndata;
  if (do_add) {
#pragma omp parallel for num_threads(ORC_THREADS(nthread)) schedule(static)
    for (int64_t i = 0; i < nn; i++) dat[i] += map[ipix[i]];
  } else {
#pragma omp parallel for num_threads(ORC_THREADS(nthread)) schedule(static)
    for (int64_t i = 0; i < nn; i++) dat[i] = map[ipix[i]];
  }
}

void orc_map2tod_serial(double *dat, const double *map, int64_t ndet,
                        int64_t ndata, const int32_t *ipix, int do_add) {
  int64_t nn = ndet * ndata;
  if (do_add)
    for (int64_t i = 0; i < nn; i++) dat[i] += map[ipix[i]];
  else
    for (int64_t i = 0; i < nn; i++) dat[i] = map[ipix[i]];
}

/* ---- tod2map: map[ipix[i]] += dat[i] ------------------------------------ */

/* Per-thread private map, static sample partition, then an ordered reduce.
 * Returns 0, or -1 if a private map could not be allocated. */
int orc_tod2map(double *map, const double *dat, int64_t ndet, int64_t ndata,
                const int32_t *ipix, int64_t npix, int nthread) {
  int nt = ORC_THREADS(nthread);
  int64_t nn = ndet * ndata;
  double *priv = (double *)calloc((size_t)nt * (size_t)npix, sizeof(double));
  if (!priv) return -1;
#pragma omp parallel num_threads(nt)
  {
    int t = omp_get_thread_num();
    double *mine = priv + (size_t)t * (size_t)npix;
#pragma omp for schedule(static)
    for (int64_t i = 0; i < nn; i++) mine[ipix[i]] += dat[i];
    /* ordered reduce: each thread owns a pixel stripe and sums the private
     * maps in thread order */
#pragma omp for schedule(static)
    for (int64_t p = 0; p < npix; p++) {
      double acc = map[p];
      for (int u = 0; u < nt; u++) acc += priv[(size_t)u * (size_t)npix + p];
      map[p] = acc;
    }
  }
  free(priv);
  return 0;
}

int orc_tod2map_f32(float *map, const float *dat, int64_t ndet, int64_t ndata,
                    const int32_t *ipix, int64_t npix, int nthread) {
  int nt = ORC_THREADS(nthread);
  int64_t nn = ndet * ndata;
  float *priv = (float *)calloc((size_t)nt * (size_t)npix, sizeof(float));
  if (!priv) return -1;
#pragma omp parallel num_threads(nt)
  {
    int t = omp_get_thread_num();
    float *mine = priv + (size_t)t * (size_t)npix;
#pragma omp for schedule(static)
    for (int64_t i = 0; i < nn; i++) mine[ipix[i]] += dat[i];
#pragma omp for schedule(static)
    for (int64_t p = 0; p < npix; p++) {
      float acc = map[p];
      for (int u = 0; u < nt; u++) acc += priv[(size_t)u * (size_t)npix + p];
      map[p] = acc;
    }
  }
  free(priv);
  return 0;
}

void orc_tod2map_serial(double *map, const double *dat, int64_t ndet,
                        int64_t ndata, const int32_t *ipix) {
  int64_t nn = ndet * ndata;
  for (int64_t i = 0; i < nn; i++) map[ipix[i]] += dat[i];
}

void orc_tod2map_atomic(double *map, const double *dat, int64_t ndet,
                        int64_t ndata, const int32_t *ipix, int nthread) {
  int64_t nn = ndet * ndata;
#pragma omp parallel for num_threads(ORC_THREADS(nthread)) schedule(static)
  for (int64_t i = 0; i < nn; i++) {
#pragma omp atomic
    map[ipix[i]] += dat[i];
  }
}

/* ---- helpers used by the PCG oracle ------------------------------------- */

/* Count of samples whose pixel index is outside [0, npix). */
int64_t orc_count_bad_pix(const int32_t *ipix, int64_t n, int64_t npix) {
  int64_t bad = 0;
#pragma omp parallel for reduction(+ : bad) schedule(static)
  for (int64_t i = 0; i < n; i++)
    if (ipix[i] < 0 || (int64_t)ipix[i] >= npix) bad++;
  return bad;
}

int orc_max_threads(void) { return omp_get_max_threads(); }
