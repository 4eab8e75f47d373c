// FP32 DCT-I by a four-step FFT in shared memory (see mk_fft4.cuh): the
// plan geometry, the twiddle tables and the FP32 kernels.  The FP64 kernels
// are mk_fft4_f64.cu (the same source, mk_fft4_kern.cuh).
#include <cufft.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <string>
#include <utility>
#include <vector>

#define MK_FFT4_NS f4s
#define MK_FFT4_C float2
#define MK_FFT4_RT float
#define MK_FFT4_FBHI 16
#define MK_FFT4_FBLO 8
#ifndef MK_FFT4_NT16
#define MK_FFT4_NT16 512
#endif
#ifndef MK_FFT4_NT8
#define MK_FFT4_NT8 512
#endif
#ifndef MK_FFT4_MINB8
#define MK_FFT4_MINB8 2
#endif
#define MK_FFT4_NTHI MK_FFT4_NT16
#define MK_FFT4_NTLO MK_FFT4_NT8
#define MK_FFT4_MINBLO MK_FFT4_MINB8
#include "mk_fft4_kern.cuh"

namespace mk {
namespace {

void factor(int64_t L, std::vector<int> &f) {
  for (int pr : {2, 3, 5, 7, 11})
    while (L % pr == 0) {
      f.push_back(pr);
      L /= pr;
    }
  if (L != 1) f.clear();
}

// radices of a transform of length Ls (a product of 2, 3, 5, 7, 11): the
// fewest stages over the radices 2 .. 16 held in registers (ties broken by
// an estimate of the arithmetic), odd ones first (the stride-1 first stage
// is then free of bank conflicts), each group in decreasing order.
// MINKASI_GB300_FFT4_RADIX=basic keeps the prime radices with 3 x 3 as 9
// and powers of 2 as 8, 4, 2.
static const int kRadix[] = {16, 15, 14, 12, 11, 10, 9, 8, 7, 6, 5, 4, 3, 2};
static const int kRadixCost[] = {4, 5, 5, 4, 6, 4, 4, 3, 4, 3, 3, 2, 2, 1};

static void radix_exps(int R, int *e) {
  const int pr[5] = {2, 3, 5, 7, 11};
  for (int i = 0; i < 5; i++) {
    e[i] = 0;
    while (R % pr[i] == 0) {
      R /= pr[i];
      e[i]++;
    }
  }
}

// best (stages, cost) radix list for the exponent vector e, memoised
struct RadixPlan {
  int stages = 1 << 20, cost = 0;
  std::vector<int> r;
};
static const RadixPlan &best_plan(const int *e, int rmax, std::vector<RadixPlan> &memo, std::vector<bool> &done) {
  const int key = (((e[0] * 8 + e[1]) * 6 + e[2]) * 5 + e[3]) * 5 + e[4];
  if (done[key]) return memo[key];
  RadixPlan best;
  if (!e[0] && !e[1] && !e[2] && !e[3] && !e[4]) {
    best.stages = 0;
  } else {
    for (size_t i = 0; i < sizeof(kRadix) / sizeof(int); i++) {
      if (kRadix[i] > rmax) continue;
      int f[5];
      radix_exps(kRadix[i], f);
      bool fits = true;
      for (int k = 0; k < 5; k++) fits &= f[k] <= e[k];
      if (!fits) continue;
      int rest[5];
      for (int k = 0; k < 5; k++) rest[k] = e[k] - f[k];
      const RadixPlan &sub = best_plan(rest, rmax, memo, done);
      const int st = sub.stages + 1, co = sub.cost + kRadixCost[i];
      if (st < best.stages || (st == best.stages && co < best.cost)) {
        best.stages = st;
        best.cost = co;
        best.r = sub.r;
        best.r.push_back(kRadix[i]);
      }
    }
  }
  memo[key] = best;
  done[key] = true;
  return memo[key];
}

bool radices(int Ls, int *r, int *nr, int rmax) {
  std::vector<int> f;
  factor(Ls, f);
  if (f.empty() && Ls != 1) return false;
  int c[12] = {0};
  for (int x : f) c[x]++;
  std::vector<int> out;
  const char *mode = getenv("MINKASI_GB300_FFT4_RADIX");
  if (mode && std::string(mode) == "basic") {
    for (int i = 0; i < c[11]; i++) out.push_back(11);
    for (; c[3] >= 2; c[3] -= 2) out.push_back(9);
    for (int i = 0; i < c[7]; i++) out.push_back(7);
    for (int i = 0; i < c[5]; i++) out.push_back(5);
    if (c[3]) out.push_back(3);
    for (; c[2] >= 3; c[2] -= 3) out.push_back(8);
    if (c[2] == 2) out.push_back(4);
    if (c[2] == 1) out.push_back(2);
  } else {
    int e[5] = {c[2], c[3], c[5], c[7], c[11]};
    if (e[0] > 10 || e[1] > 7 || e[2] > 5 || e[3] > 4 || e[4] > 4) return false;
    std::vector<RadixPlan> memo(11 * 8 * 6 * 5 * 5);
    std::vector<bool> done(memo.size(), false);
    out = best_plan(e, rmax, memo, done).r;
    std::stable_sort(out.begin(), out.end(), [](int a, int b) {
      if ((a & 1) != (b & 1)) return (a & 1) > (b & 1);
      return a > b;
    });
  }
  if ((int)out.size() > FFT4_MAXR) return false;
  for (size_t i = 0; i < out.size(); i++) r[i] = out[i];
  *nr = (int)out.size();
  return true;
}

size_t al(size_t x) { return (x + 255) / 256 * 256; }

struct TableLayout {
  size_t stw1, stw2, iperm1, iperm2, tlane, tblk, chirp, bhat, tlane2, tblk2, total;
};

size_t csz(const Fft4Dev &d);

TableLayout layout(const Fft4Dev &d) {
  TableLayout t;
  size_t o = 0;
  t.stw1 = o;
  o += al((size_t)d.L1 * csz(d));
  t.stw2 = o;
  o += al((size_t)d.L2 * csz(d));
  t.iperm1 = o;
  o += al((size_t)d.L1 * sizeof(int));
  t.iperm2 = o;
  o += al((size_t)d.L2 * sizeof(int));
  t.tlane = o;
  o += al((size_t)d.L1 * 32 * csz(d));
  t.tblk = o;
  o += al((size_t)d.L1 * d.nb32 * csz(d));
  t.chirp = o;
  o += d.blue ? al((size_t)(d.m + 1) * csz(d)) : 0;
  t.bhat = o;
  o += d.blue ? al((size_t)d.L * csz(d)) : 0;
  t.tlane2 = o;
  o += d.blue ? al((size_t)d.L2 * 32 * csz(d)) : 0;
  t.tblk2 = o;
  o += d.blue ? al((size_t)d.L2 * ((d.L1 + 31) / 32) * csz(d)) : 0;
  t.total = o;
  return t;
}

struct Cd {
  double x, y;
};

Cd unit(double num, double den) {
  // exp(-2 pi i num / den) in double
  const double a = 2.0 * M_PI * num / den;
  return {std::cos(a), -std::sin(a)};
}

// a complex table entry at byte offset `off`, index i: float2 or double2
void put(char *base, size_t off, int64_t i, Cd v, bool f64) {
  if (f64) {
    reinterpret_cast<double2 *>(base + off)[i] = make_double2(v.x, v.y);
  } else {
    reinterpret_cast<float2 *>(base + off)[i] = make_float2((float)v.x, (float)v.y);
  }
}

size_t csz(const Fft4Dev &d) { return d.f64 ? sizeof(double2) : csz(d); }

void digit_rev(int Ls, const int *r, int nr, int *P) {
  std::vector<int> d(nr > 0 ? nr : 1);
  for (int j = 0; j < Ls; j++) {
    int q = j;
    for (int i = nr - 1; i >= 0; i--) {
      d[i] = q % r[i];
      q /= r[i];
    }
    int pos = 0, span = 1;
    for (int i = 0; i < nr; i++) {
      pos += d[i] * span;
      span *= r[i];
    }
    P[j] = pos;
  }
}

}  // namespace

// Which L1 x L2 split new plans take: 0 = the divisor pair closest to
// sqrt(L), r = the r-th next closest (the last one when there are fewer).
// Set by the autotuner around plan creation; a plan keeps its split.
static std::atomic<int> g_split_rank{0};
void fft4_set_split_rank(int r) { g_split_rank.store(r < 0 ? 0 : r); }
int fft4_split_rank() { return g_split_rank.load(); }

// L1 x L2 split of a transform of length L (by g_split_rank among the
// divisor pairs with both parts <= LMAX and L1 > 1, ordered by closeness to
// sqrt(L)), radices and stage constants
static bool split_len(int64_t L, Fft4Dev *t) {
  if (L < 2 || L > (int64_t)FFT4_LMAX * FFT4_LMAX) return false;
  std::vector<int> f;
  factor(L, f);
  if (f.empty()) return false;
  std::vector<int64_t> ds{1};
  for (int pr : f) {
    const size_t k = ds.size();
    for (size_t i = 0; i < k; i++) {
      const int64_t v = ds[i] * pr;
      bool seen = false;
      for (int64_t u : ds) seen |= (u == v);
      if (!seen) ds.push_back(v);
    }
  }
  std::vector<std::pair<double, int64_t>> cand;
  for (int64_t a : ds) {
    const int64_t b = L / a;
    if (a > FFT4_LMAX || b > FFT4_LMAX || a == 1) continue;  // pass B needs at least one stage
    cand.push_back({std::fabs(std::log((double)a) - std::log((double)b)), a});
  }
  if (cand.empty()) return false;
  std::sort(cand.begin(), cand.end());
  const size_t rank = (size_t)g_split_rank.load();
  const int64_t best = cand[rank < cand.size() ? rank : cand.size() - 1].second;
  t->L = L;
  t->L1 = (int)best;
  t->L2 = (int)(L / best);
  const int rmax = t->f64 ? MK_FFT4_RMAX64 : MK_FFT4_RMAX;
  if (!radices(t->L1, t->r1, &t->nr1, rmax) || !radices(t->L2, t->r2, &t->nr2, rmax)) return false;
  t->nb32 = (t->L2 + 31) / 32;
  for (int pass = 0; pass < 2; pass++) {
    const int nr = pass ? t->nr2 : t->nr1;
    const int *r = pass ? t->r2 : t->r1;
    int *ns = pass ? t->ns2 : t->ns1, *to = pass ? t->to2 : t->to1;
    float *inv = pass ? t->inv2 : t->inv1;
    int span = 1, off = 0;
    for (int s = 0; s < nr; s++) {
      ns[s] = span;
      to[s] = off;
      inv[s] = 1.0f / (float)span;
      off += (r[s] - 1) * span;
      span *= r[s];
    }
  }
  return true;
}

// transforms per CTA for a pass of length Ls: the wide tile (16 in FP32, 8
// in FP64: wider coalesced rows) while two such CTAs fit in an SM's shared
// memory, else half of it.  MINKASI_GB300_FFT4_FB=lo or hi forces one.
static int fb_for(int Ls, bool f64) {
  const int hi = f64 ? 8 : 16, lo = hi / 2;
  const char *e = getenv("MINKASI_GB300_FFT4_FB");
  if (e && std::string(e) == "lo") return lo;
  if (e && std::string(e) == "hi") return hi;
  return hi * (size_t)(Ls | 1) * (f64 ? sizeof(double2) : sizeof(float2)) <= 113 * 1024 ? hi : lo;
}

bool fft4_shape(int64_t n, Fft4Dev *d, bool bluestein, bool f64) {
  if (n < 2 || n > (int64_t)FFT4_LMAX * FFT4_LMAX / 2) return false;
  Fft4Dev t{};
  t.f64 = f64;
  t.n = n;
  t.m = n - 1;
  t.Lx = 2 * t.m;
  bool ok = false;
  if (split_len(t.Lx, &t)) {
    t.blue = false;
    ok = true;
  } else if (bluestein) {
    for (int64_t M = 3 * t.m; M <= (int64_t)FFT4_LMAX * FFT4_LMAX && !ok; M++) {
      if (split_len(M, &t)) {
        t.blue = true;
        ok = true;
      }
    }
  }
  if (!ok) return false;
  t.fba = fb_for(t.L2, f64);
  t.fbb = fb_for(t.L1, f64);
  // MINKASI_GB300_FFT4_BLUE3=0 makes new Bluestein plans keep the four-pass form
  const char *e4 = getenv("MINKASI_GB300_FFT4_BLUE3");
  t.blue4 = t.blue && e4 && std::string(e4) == "0";
  *d = t;
  return true;
}

size_t fft4_table_bytes(const Fft4Dev &d) { return layout(d).total; }

size_t fft4_t_bytes(const Fft4Dev &d, int64_t nrow) {
  return (d.blue ? 2 : 1) * (size_t)((nrow + 1) / 2) * (size_t)d.L * csz(d);
}

// B^ = DFT_M(b) / M with b_t = conj(c_t) at t mod M for t in [-m, 2m - 1]
// (M >= 3m keeps those positions distinct), in double precision through a
// cuFFT Z2Z transform, rounded to the plan's precision
static int bluestein_bhat(const Fft4Dev &d, char *base, size_t off) {
  const int64_t M = d.L, Lx = d.Lx, m = d.m;
  std::vector<cufftDoubleComplex> b((size_t)M);
  for (auto &v : b) v.x = v.y = 0.0;
  for (int64_t t = 0; t < 2 * m; t++) {
    const double a = M_PI * (double)((t * t) % (2 * Lx)) / (double)Lx;  // conj(c_t) = exp(+i a)
    b[(size_t)t].x = std::cos(a);
    b[(size_t)t].y = std::sin(a);
    if (t > 0 && t <= m) b[(size_t)(M - t)] = b[(size_t)t];
  }
  cufftDoubleComplex *db = nullptr;
  MK_CUDA(cudaMalloc(&db, (size_t)M * sizeof(cufftDoubleComplex)));
  int rc = MK_OK;
  cufftHandle h = 0;
  if (cudaMemcpy(db, b.data(), (size_t)M * sizeof(cufftDoubleComplex), cudaMemcpyHostToDevice) != cudaSuccess ||
      cufftPlan1d(&h, (int)M, CUFFT_Z2Z, 1) != CUFFT_SUCCESS ||
      cufftExecZ2Z(h, db, db, CUFFT_FORWARD) != CUFFT_SUCCESS ||
      cudaMemcpy(b.data(), db, (size_t)M * sizeof(cufftDoubleComplex), cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error("fft4: Bluestein kernel transform (M = %lld) failed", (long long)M);
    rc = MK_ERR_CUFFT;
  }
  if (h) cufftDestroy(h);
  cudaFree(db);
  if (rc) return rc;
  for (int64_t k = 0; k < M; k++)
    put(base, off, k, {b[(size_t)k].x / (double)M, b[(size_t)k].y / (double)M}, d.f64);
  return MK_OK;
}

int fft4_init(Fft4Plan *p, int64_t n, void *dev_tables, bool bluestein, bool f64) {
  MK_CHECK_ARG(fft4_shape(n, &p->d, bluestein, f64), "fft4: row length %lld has no supported factorisation",
               (long long)n);
  Fft4Dev &d = p->d;
  const TableLayout t = layout(d);
  std::vector<char> h(t.total, 0);
  for (int pass = 0; pass < 2; pass++) {
    const int nr = pass ? d.nr2 : d.nr1;
    const int *r = pass ? d.r2 : d.r1, *ns = pass ? d.ns2 : d.ns1, *to = pass ? d.to2 : d.to1;
    const size_t so = pass ? t.stw2 : t.stw1;
    for (int s = 0; s < nr; s++)
      for (int rr = 1; rr < r[s]; rr++)
        for (int k = 0; k < ns[s]; k++)
          put(h.data(), so, to[s] + (rr - 1) * ns[s] + k, unit((double)rr * k, (double)ns[s] * r[s]), d.f64);
  }
  {
    std::vector<int> P1(d.L1), P2(d.L2);
    digit_rev(d.L1, d.r1, d.nr1, P1.data());
    digit_rev(d.L2, d.r2, d.nr2, P2.data());
    int *I1 = (int *)(h.data() + t.iperm1), *I2 = (int *)(h.data() + t.iperm2);
    for (int j = 0; j < d.L1; j++) I1[P1[j]] = j;
    for (int j = 0; j < d.L2; j++) I2[P2[j]] = j;
  }
  for (int64_t j1 = 0; j1 < d.L1; j1++) {
    for (int l = 0; l < 32; l++) put(h.data(), t.tlane, 32 * j1 + l, unit((double)(j1 * l % d.L), (double)d.L), d.f64);
    for (int i = 0; i < d.nb32; i++)
      put(h.data(), t.tblk, j1 * d.nb32 + i, unit((double)(j1 * 32 * i % d.L), (double)d.L), d.f64);
  }
  if (d.blue) {
    for (int64_t j = 0; j <= d.m; j++)
      put(h.data(), t.chirp, j, unit((double)((j * j) % (2 * d.Lx)), 2.0 * (double)d.Lx), d.f64);
    const int rc = bluestein_bhat(d, h.data(), t.bhat);
    if (rc) return rc;
    d.nb32b = (d.L1 + 31) / 32;
    for (int64_t k2 = 0; k2 < d.L2; k2++) {
      for (int l = 0; l < 32; l++)
        put(h.data(), t.tlane2, 32 * k2 + l, unit((double)(k2 * l % d.L), (double)d.L), d.f64);
      for (int i = 0; i < d.nb32b; i++)
        put(h.data(), t.tblk2, k2 * d.nb32b + i, unit((double)(k2 * 32 * i % d.L), (double)d.L), d.f64);
    }
  }
  MK_CUDA(cudaMemcpy(dev_tables, h.data(), t.total, cudaMemcpyHostToDevice));
  char *b = (char *)dev_tables;
  d.stw1 = (const void *)(b + t.stw1);
  d.stw2 = (const void *)(b + t.stw2);
  d.iperm1 = (const int *)(b + t.iperm1);
  d.iperm2 = (const int *)(b + t.iperm2);
  d.tlane = (const void *)(b + t.tlane);
  d.tblk = (const void *)(b + t.tblk);
  d.chirp = d.blue ? (const void *)(b + t.chirp) : nullptr;
  d.bhat = d.blue ? (const void *)(b + t.bhat) : nullptr;
  d.tlane2 = d.blue ? (const void *)(b + t.tlane2) : nullptr;
  d.tblk2 = d.blue ? (const void *)(b + t.tblk2) : nullptr;
  p->tables = dev_tables;
  return MK_OK;
}


int fft4_dct(const Fft4Plan &p, const float *x, int64_t ldx, int64_t nrow, float2 *T, float *out, int64_t ldo,
             int epi, const float *w, int64_t ldw, cudaStream_t st) {
  return f4s::dct_launch(p, x, ldx, nrow, T, out, ldo, epi, w, ldw, st);
}

}  // namespace mk
