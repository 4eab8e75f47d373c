// 3x3 convolutions for the learned SPD map-space preconditioner
//   M = D^-1/2 (I + K^T K) D^-1/2,  K = L4 L3 L2 L1 (linear 3x3 convolutions)
// applied to map-sized PCG residuals.  Three kernels cover inference and
// training:
//   conv_fwd : Y[b,co,p]  = sum_ci sum_d W[co,ci,d] X[b,ci,p+d]       (L x)
//   conv_adj : X[b,ci,q]  = sum_co sum_d W[co,ci,d] Y[b,co,q-d]       (L^T y)
//   conv_wgrad: G[co,ci,d] = sum_b sum_p H[b,co,p] X[b,ci,p+d]
// with zero padding (pixels outside the map are 0).  Layout: [B][C][H][W],
// FP32, at most 16 channels.  Each CTA stages its input tile plus a 1-pixel
// halo for every channel in shared memory, and the weights (<= 16*16*9
// floats) are read as warp-wide broadcasts; threads are register-blocked
// (see k_conv and k_conv_wgrad).  conv_wgrad writes one partial per CTA and a
// second kernel sums the partials in a fixed order (reproducible gradients).
#include "mk_async.cuh"
#include "mk_common.cuh"

namespace {

constexpr int CMAX = 16;
constexpr int NW = CMAX * CMAX * 9;

// ---- fwd / adjoint: one kernel, register-blocked ------------------------
// A CTA owns a TXT x TYT tile of output pixels; each thread a 1x4 strip of it
// for NOUT / OG of the output channels (OG threads share a strip, one warp
// all on the same channel group).  The weights of one input channel and tap
// are contiguous over the output channels, so one 16-byte shared-memory load
// brings 4 of them, each feeding 4 FMAs.  The input tile plus a 1-pixel halo
// is staged in shared memory for every input channel with asynchronous
// 4-byte copies (zero-filled outside the map), all in flight at once.  The
// adjoint is the same loop with input and output channels swapped and the
// taps flipped:  adj(o = ci, i = co, d) = W[co][ci][8 - d].
// Large maps use 32 x 32 tiles with one thread per strip (256 threads);
// small ones 16 x 16 tiles with 4 channel groups (256 threads), which gives
// the GPU 4x as many warps for the same work.
constexpr int PX = 4;

template <int TXT, int TYT, int OG>
struct Tile {
  static constexpr int SXW = TXT + 2, SXH = TYT + 2, NS = (TXT / PX) * TYT, NT = NS * OG;
};

// input planes, then the weights as [ci][tap][o] with o padded to NOUT
template <int TXT, int TYT>
size_t conv_smem(int nin, int nout_t) {
  return ((size_t)nin * Tile<TXT, TYT, 1>::SXH * Tile<TXT, TYT, 1>::SXW + (size_t)nin * 9 * nout_t) *
         sizeof(float);
}

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// EPI selects what surrounds the convolution (TT = the map type, float or
// double): 0 plain FP32 in/out; 1 the single input plane is u = dsq * r,
// formed while staging (In unused); 2 the single output plane is written as
// z = dsq * (dsq * r + conv) (Out unused).  1 and 2 are the first and last
// layers of the preconditioner M r = D^-1/2 (u + K^T K u), u = D^-1/2 r.
template <bool ADJ, int NOUT, int OG, int TXT, int TYT, int EPI = 0, typename TT = float>
__global__ void __launch_bounds__(Tile<TXT, TYT, OG>::NT)
    k_conv(const float *__restrict__ In, const float *__restrict__ Wt, float *__restrict__ Out, int Cin, int Cout,
           int H, int W, const TT *__restrict__ r, const TT *__restrict__ dsq, TT *__restrict__ z) {
  using T = Tile<TXT, TYT, OG>;
  constexpr int SXW = T::SXW, SXH = T::SXH, NT = T::NT, NO = NOUT / OG;
  static_assert(NOUT % OG == 0 && (OG == 1 || NO % 4 == 0), "channel groups of 4");
  extern __shared__ float smem[];
  const int nin = ADJ ? Cout : Cin, nout = ADJ ? Cin : Cout;
  float *sx = smem;
  float *sw = smem + nin * SXH * SXW;
  const int b = blockIdx.z, y0 = blockIdx.y * TYT, x0 = blockIdx.x * TXT, tid = threadIdx.x;
  if constexpr (EPI == 1) {
    // nin == 1
    for (int i = tid; i < SXH * SXW; i += NT) {
      const int yy = y0 + i / SXW - 1, xx = x0 + i % SXW - 1;
      float v = 0.f;
      if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
        const int64_t g = ((int64_t)b * H + yy) * W + xx;
        v = (float)mul_rn(dsq[g], r[g]);
      }
      sx[i] = v;
    }
  } else {
    const float *ib = In + (int64_t)b * nin * H * W;
    for (int i = tid; i < nin * SXH * SXW; i += NT) {
      const int c = i / (SXH * SXW), rr = (i / SXW) % SXH, q = i % SXW;
      const int yy = y0 + rr - 1, xx = x0 + q - 1;
      const bool ok = yy >= 0 && yy < H && xx >= 0 && xx < W;
      mk::cp_async4_zfill(sx + i, ok ? ib + (int64_t)c * H * W + (int64_t)yy * W + xx : ib, ok);
    }
  }
  for (int i = tid; i < nin * 9 * NOUT; i += NT) {
    const int o = i % NOUT, d = (i / NOUT) % 9, ii = i / (9 * NOUT);
    sw[i] = o >= nout ? 0.f : ADJ ? Wt[(ii * Cin + o) * 9 + (8 - d)] : Wt[(o * Cin + ii) * 9 + d];
  }
  mk::cp_async_wait_all();
  __syncthreads();
  const int strip = tid % T::NS, o0 = (tid / T::NS) * NO;
  const int ty = strip / (TXT / PX), tx = (strip % (TXT / PX)) * PX;
  float acc[PX][NO];
#pragma unroll
  for (int p = 0; p < PX; p++)
#pragma unroll
    for (int o = 0; o < NO; o++) acc[p][o] = 0.f;
  for (int ci = 0; ci < nin; ci++) {
    const float *sp = sx + ci * SXH * SXW + ty * SXW + tx;
    float win[3][PX + 2];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int c = 0; c < PX + 2; c++) win[r][c] = sp[r * SXW + c];
    const float *wc = sw + ci * 9 * NOUT + o0;
#pragma unroll
    for (int d = 0; d < 9; d++) {
      float wv[NO];
      if constexpr (NO % 4 == 0) {
#pragma unroll
        for (int k = 0; k < NO / 4; k++) {
          const float4 q = reinterpret_cast<const float4 *>(wc + d * NOUT)[k];
          wv[4 * k] = q.x, wv[4 * k + 1] = q.y, wv[4 * k + 2] = q.z, wv[4 * k + 3] = q.w;
        }
      } else {
#pragma unroll
        for (int o = 0; o < NO; o++) wv[o] = wc[d * NOUT + o];
      }
#pragma unroll
      for (int o = 0; o < NO; o++)
#pragma unroll
        for (int p = 0; p < PX; p++) acc[p][o] = fmaf(wv[o], win[d / 3][p + d % 3], acc[p][o]);
    }
  }
  const int yy = y0 + ty;
  if (yy >= H) return;
  if constexpr (EPI == 2) {
    // nout == 1
    if (o0 != 0) return;
#pragma unroll
    for (int p = 0; p < PX; p++) {
      const int xx = x0 + tx + p;
      if (xx < W) {
        const int64_t g = ((int64_t)b * H + yy) * W + xx;
        const TT d = dsq[g];
        z[g] = mul_rn(d, add_rn(mul_rn(d, r[g]), (TT)acc[p][0]));
      }
    }
    return;
  }
  float *ob = Out + (int64_t)b * nout * H * W + (int64_t)yy * W;
#pragma unroll
  for (int p = 0; p < PX; p++) {
    const int xx = x0 + tx + p;
    if (xx < W) {
#pragma unroll
      for (int o = 0; o < NO; o++)
        if (o0 + o < nout) ob[(int64_t)(o0 + o) * H * W + xx] = acc[p][o];
    }
  }
}

// ---- weight gradient -----------------------------------------------------
// G[co][ci][d] = sum_p H[co, p] X[ci, p + d] over a 16x32 pixel tile per CTA.
// Thread (rowgroup, co-group, ci) keeps 4 output channels x 9 taps in
// registers and slides a 3x3 window of X along its 4 rows: per pixel 3 new X
// values and 4 H values feed 36 FMAs.  Shared-memory planes are padded so
// that the 16 input channels (and the 8 output channels) a warp reads at once
// fall in distinct banks.  The 4 row groups are summed in a fixed order and
// each CTA writes one partial; k_wgrad_reduce sums the partials in CTA order.
constexpr int WTX = 32, WTY = 16;
constexpr int XPL = (WTY + 2) * (WTX + 2) + 1;  // X plane stride (mod 32 = 5)
constexpr int HPL = WTY * WTX + 1;              // H plane stride (mod 32 = 1)

__global__ void __launch_bounds__(256) k_conv_wgrad(const float *__restrict__ X, const float *__restrict__ Hg,
                                                    float *__restrict__ part, int Cin, int Cout, int H, int W) {
  extern __shared__ float smem[];
  float *sx = smem;                 // [CMAX][XPL]
  float *sh = smem + CMAX * XPL;    // [CMAX][HPL]
  float *red = sh + CMAX * HPL;     // [4][NW]
  const int b = blockIdx.z, y0 = blockIdx.y * WTY, x0 = blockIdx.x * WTX, tid = threadIdx.x;
  const float *xb = X + (int64_t)b * Cin * H * W;
  const float *hb = Hg + (int64_t)b * Cout * H * W;
  for (int i = tid; i < Cin * (WTY + 2) * (WTX + 2); i += 256) {
    const int c = i / ((WTY + 2) * (WTX + 2)), rq = i % ((WTY + 2) * (WTX + 2));
    const int yy = y0 + rq / (WTX + 2) - 1, xx = x0 + rq % (WTX + 2) - 1;
    const bool ok = yy >= 0 && yy < H && xx >= 0 && xx < W;
    mk::cp_async4_zfill(sx + c * XPL + rq, ok ? xb + (int64_t)c * H * W + (int64_t)yy * W + xx : xb, ok);
  }
  for (int i = tid; i < Cout * WTY * WTX; i += 256) {
    const int c = i / (WTY * WTX), rq = i % (WTY * WTX);
    const int yy = y0 + rq / WTX, xx = x0 + rq % WTX;
    const bool ok = yy < H && xx < W;
    mk::cp_async4_zfill(sh + c * HPL + rq, ok ? hb + (int64_t)c * H * W + (int64_t)yy * W + xx : hb, ok);
  }
  mk::cp_async_wait_all();
  __syncthreads();
  const int ci = tid & 15, cg = (tid >> 4) & 3, rg = tid >> 6;  // 16 ci x 4 co-groups x 4 row groups
  float acc[4][9];
#pragma unroll
  for (int k = 0; k < 4; k++)
#pragma unroll
    for (int d = 0; d < 9; d++) acc[k][d] = 0.f;
  if (ci < Cin && cg * 4 < Cout) {
    for (int r = rg * (WTY / 4); r < (rg + 1) * (WTY / 4); r++) {
      const float *xp = sx + ci * XPL + r * (WTX + 2);
      float win[3][3];
#pragma unroll
      for (int dy = 0; dy < 3; dy++) {
        win[dy][1] = xp[dy * (WTX + 2) + 0];
        win[dy][2] = xp[dy * (WTX + 2) + 1];
      }
      for (int q = 0; q < WTX; q++) {
#pragma unroll
        for (int dy = 0; dy < 3; dy++) {
          win[dy][0] = win[dy][1];
          win[dy][1] = win[dy][2];
          win[dy][2] = xp[dy * (WTX + 2) + q + 2];
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
          const int co = cg * 4 + k;
          const float h = co < Cout ? sh[co * HPL + r * WTX + q] : 0.f;
#pragma unroll
          for (int d = 0; d < 9; d++) acc[k][d] = fmaf(h, win[d / 3][d % 3], acc[k][d]);
        }
      }
    }
  }
  const int nw = Cout * Cin * 9;
  if (ci < Cin) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const int co = cg * 4 + k;
      if (co < Cout)
#pragma unroll
        for (int d = 0; d < 9; d++) red[rg * NW + (co * Cin + ci) * 9 + d] = acc[k][d];
    }
  }
  __syncthreads();
  const int64_t cta = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  for (int w = tid; w < nw; w += 256)
    part[cta * nw + w] = (red[w] + red[NW + w]) + (red[2 * NW + w] + red[3 * NW + w]);
}

constexpr size_t WGRAD_SMEM = (size_t)(CMAX * XPL + CMAX * HPL + 4 * NW) * sizeof(float);

// G[w] = sum over CTAs of part[cta][w], in CTA order (reproducible)
__global__ void k_wgrad_reduce(const float *__restrict__ part, int64_t ncta, int nw, float *__restrict__ G) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  double acc = 0.0;
  for (int64_t c = 0; c < ncta; c++) acc += (double)part[c * nw + w];
  G[w] = (float)acc;
}

int conv_args(int B, int Cin, int Cout, int H, int W) {
  MK_CHECK_ARG(B >= 1 && H >= 1 && W >= 1, "conv: bad shape B=%d H=%d W=%d", B, H, W);
  MK_CHECK_ARG(Cin >= 1 && Cin <= CMAX && Cout >= 1 && Cout <= CMAX,
               "conv: channels must be in [1, %d] (got %d -> %d)", CMAX, Cin, Cout);
  MK_CHECK_ARG(B <= 65535, "conv: batch too large");
  return MK_OK;
}

dim3 wgrad_grid(int B, int H, int W) { return dim3((W + WTX - 1) / WTX, (H + WTY - 1) / WTY, B); }

template <bool ADJ, int OG, int TXT, int TYT, int EPI, typename TT>
int conv_launch_t(const float *in, const float *w, float *out, int B, int Cin, int Cout, int H, int W,
                  const TT *r, const TT *dsq, TT *z, cudaStream_t st, const char *what) {
  static bool attr[64] = {false};
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  const int nin = ADJ ? Cout : Cin, nout = ADJ ? Cin : Cout;
  const size_t smem = conv_smem<TXT, TYT>(nin, nout == 1 ? 1 : CMAX);
  auto k16 = k_conv<ADJ, CMAX, OG, TXT, TYT, EPI, TT>;
  auto k1 = k_conv<ADJ, 1, 1, TXT, TYT, EPI, TT>;
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    const int mx = (int)conv_smem<TXT, TYT>(CMAX, CMAX);
    if constexpr (EPI != 2) MK_CUDA(cudaFuncSetAttribute(k16, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    MK_CUDA(cudaFuncSetAttribute(k1, cudaFuncAttributeMaxDynamicSharedMemorySize, mx));
    attr[dev] = true;
  }
  dim3 g((W + TXT - 1) / TXT, (H + TYT - 1) / TYT, B);
  if constexpr (EPI == 2) {
    k1<<<g, Tile<TXT, TYT, 1>::NT, smem, st>>>(in, w, out, Cin, Cout, H, W, r, dsq, z);
  } else {
    if (nout == 1)
      k1<<<g, Tile<TXT, TYT, 1>::NT, smem, st>>>(in, w, out, Cin, Cout, H, W, r, dsq, z);
    else
      k16<<<g, Tile<TXT, TYT, OG>::NT, smem, st>>>(in, w, out, Cin, Cout, H, W, r, dsq, z);
  }
  return mk::launch_status(what);
}

// 32 x 32 tiles when they give every SM at least 4; 16 x 16 with 4 channel
// groups otherwise
template <bool ADJ, int EPI = 0, typename TT = float>
int conv_launch(const float *in, const float *w, float *out, int B, int Cin, int Cout, int H, int W,
                cudaStream_t st, const char *what, const TT *r = nullptr, const TT *dsq = nullptr,
                TT *z = nullptr) {
  const int64_t big_tiles = (int64_t)((W + 31) / 32) * ((H + 31) / 32) * B;
  if (big_tiles >= 4LL * mk::sm_count())
    return conv_launch_t<ADJ, 1, 32, 32, EPI, TT>(in, w, out, B, Cin, Cout, H, W, r, dsq, z, st, what);
  return conv_launch_t<ADJ, 4, 16, 16, EPI, TT>(in, w, out, B, Cin, Cout, H, W, r, dsq, z, st, what);
}

template <typename TT>
int precon_apply(TT *z, const TT *r, const TT *dsq, int H, int W, int nl, const int *ch, const float *const *wt,
                 float *work, int maxc, cudaStream_t st) {
  float *buf[2] = {work, work + (size_t)maxc * H * W};
  const char *what = "mk_learned_precon_apply";
  int cur = 0;
  int rc = conv_launch<false, 1, TT>(nullptr, wt[0], buf[0], 1, 1, ch[1], H, W, st, what, r, dsq, nullptr);
  for (int l = 1; l < nl && !rc; l++, cur ^= 1)
    rc = conv_launch<false>(buf[cur], wt[l], buf[cur ^ 1], 1, ch[l], ch[l + 1], H, W, st, what);
  for (int l = nl - 1; l >= 1 && !rc; l--, cur ^= 1)
    rc = conv_launch<true>(buf[cur], wt[l], buf[cur ^ 1], 1, ch[l], ch[l + 1], H, W, st, what);
  if (!rc) rc = conv_launch<true, 2, TT>(buf[cur], wt[0], nullptr, 1, 1, ch[1], H, W, st, what, r, dsq, z);
  return rc;
}

// ---- the preconditioner as one stencil -----------------------------------
// The layers are linear and shift-invariant, so K^T K is one single-channel
// convolution whose kernel C is its impulse response, of half-width 2n for n
// 3x3 layers (17 x 17 for 4 layers).  One kernel then applies
//   z = dsq * (u + C * u),  u = dsq * r
// reading each r and dsq once.  A CTA owns a 32 x 32 output tile: u for the
// tile plus a HALF-pixel halo is staged in shared memory (zero outside the
// map) at an odd-by-one pitch, so the 4 rows a warp touches fall on distinct
// banks; each thread accumulates a 1 x 4 strip, with the KS + 3 input values
// of a stencil row in registers and C read as warp-wide broadcasts.
constexpr int ST_TX = 32, ST_TY = 32, ST_THREADS = 256, ST_MAXHALF = 8;

// PLAIN: the coarse-grid form of the pooled preconditioner, u = r and
// z = C * u (no D^-1/2, no identity term); dsq is unused.
template <int HALF, typename TT, bool PLAIN = false>
__global__ void __launch_bounds__(ST_THREADS)
    k_precon_stencil(const TT *__restrict__ r, const TT *__restrict__ dsq, const float *__restrict__ kern,
                     TT *__restrict__ z, int H, int W) {
  constexpr int KS = 2 * HALF + 1, SW = ST_TX + 2 * HALF, SH = ST_TY + 2 * HALF, P = SW | 1;
  constexpr int PITCH = (P % 4 == 1) ? P : P + 2;  // == 1 (mod 4): the 4 rows of a warp hit distinct banks
  __shared__ float su[SH * PITCH];
  __shared__ float sk[KS * KS];
  const int x0 = blockIdx.x * ST_TX, y0 = blockIdx.y * ST_TY, tid = threadIdx.x;
  for (int i = tid; i < KS * KS; i += ST_THREADS) sk[i] = kern[i];
  for (int i = tid; i < SH * SW; i += ST_THREADS) {
    const int sy = i / SW, sx = i - sy * SW, yy = y0 + sy - HALF, xx = x0 + sx - HALF;
    float v = 0.f;
    if (yy >= 0 && yy < H && xx >= 0 && xx < W) {
      const int64_t g = (int64_t)yy * W + xx;
      v = PLAIN ? (float)r[g] : (float)mul_rn(dsq[g], r[g]);
    }
    su[sy * PITCH + sx] = v;
  }
  __syncthreads();
  const int ty = tid >> 3, tx = (tid & 7) * 4;
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
  for (int dy = 0; dy < KS; dy++) {
    float row[KS + 3];
    const float *src = su + (ty + dy) * PITCH + tx;
#pragma unroll
    for (int j = 0; j < KS + 3; j++) row[j] = src[j];
    const float *kr = sk + dy * KS;
#pragma unroll
    for (int dx = 0; dx < KS; dx++) {
      const float k = kr[dx];
#pragma unroll
      for (int o = 0; o < 4; o++) acc[o] = fmaf(k, row[o + dx], acc[o]);
    }
  }
  const int yy = y0 + ty;
  if (yy >= H) return;
#pragma unroll
  for (int o = 0; o < 4; o++) {
    const int xx = x0 + tx + o;
    if (xx < W) {
      const int64_t g = (int64_t)yy * W + xx;
      if (PLAIN) {
        z[g] = (TT)acc[o];
      } else {
        const TT u = mul_rn(dsq[g], r[g]);
        z[g] = mul_rn(dsq[g], add_rn(u, (TT)acc[o]));
      }
    }
  }
}

template <int HALF, typename TT, bool PLAIN = false>
int stencil_launch(TT *z, const TT *r, const TT *dsq, const float *kern, int H, int W, cudaStream_t st) {
  const dim3 grid((W + ST_TX - 1) / ST_TX, (H + ST_TY - 1) / ST_TY);
  k_precon_stencil<HALF, TT, PLAIN><<<grid, ST_THREADS, 0, st>>>(r, dsq, kern, z, H, W);
  return mk::launch_status("mk_learned_precon_stencil");
}

template <typename TT, bool PLAIN = false>
int stencil_dispatch(TT *z, const TT *r, const TT *dsq, const float *kern, int H, int W, int half,
                     cudaStream_t st) {
  switch (half) {
    case 0: return stencil_launch<0, TT, PLAIN>(z, r, dsq, kern, H, W, st);
    case 1: return stencil_launch<1, TT, PLAIN>(z, r, dsq, kern, H, W, st);
    case 2: return stencil_launch<2, TT, PLAIN>(z, r, dsq, kern, H, W, st);
    case 3: return stencil_launch<3, TT, PLAIN>(z, r, dsq, kern, H, W, st);
    case 4: return stencil_launch<4, TT, PLAIN>(z, r, dsq, kern, H, W, st);
    case 5: return stencil_launch<5, TT, PLAIN>(z, r, dsq, kern, H, W, st);
    case 6: return stencil_launch<6, TT, PLAIN>(z, r, dsq, kern, H, W, st);
    case 7: return stencil_launch<7, TT, PLAIN>(z, r, dsq, kern, H, W, st);
    default: return stencil_launch<8, TT, PLAIN>(z, r, dsq, kern, H, W, st);
  }
}

// ---- the pooled (multi-scale) form ------------------------------------------
//   M r = dsq * (u + P^T C * P u),  u = dsq * r,
// P the b x b block mean onto an Hc x Wc grid (Hc = ceil(H / b); pixels
// outside the map count as 0) and P^T its transpose (each fine pixel gets its
// block's value / b^2).  The network then acts at b times the pixel scale,
// so its footprint is b (4n + 1) fine pixels; M stays symmetric positive
// definite.  Three launches: pool, the plain stencil on the coarse grid,
// and the unpool with the identity term and both D^-1/2 scalings.
template <typename TT>
__global__ void __launch_bounds__(256) k_pool(const TT *__restrict__ r, const TT *__restrict__ dsq,
                                              float *__restrict__ uc, int H, int W, int b, int Hc, int Wc) {
  const int64_t n = (int64_t)Hc * Wc;
  const float inv = 1.0f / (float)(b * b);
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (int64_t)gridDim.x * blockDim.x) {
    const int I = (int)(c / Wc), J = (int)(c - (int64_t)I * Wc);
    float acc = 0.f;
    for (int di = 0; di < b; di++) {
      const int i = I * b + di;
      if (i >= H) break;
      for (int dj = 0; dj < b; dj++) {
        const int j = J * b + dj;
        if (j >= W) break;
        const int64_t g = (int64_t)i * W + j;
        acc += (float)mul_rn(dsq[g], r[g]);
      }
    }
    uc[c] = acc * inv;
  }
}

template <typename TT>
__global__ void __launch_bounds__(256) k_unpool(const TT *__restrict__ r, const TT *__restrict__ dsq,
                                                const float *__restrict__ wc, TT *__restrict__ z, int H, int W,
                                                int b, int Wc) {
  const int64_t n = (int64_t)H * W;
  const float inv = 1.0f / (float)(b * b);
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(g / W), j = (int)(g - (int64_t)i * W);
    const TT u = mul_rn(dsq[g], r[g]);
    const TT w = (TT)(wc[(int64_t)(i / b) * Wc + j / b] * inv);
    z[g] = mul_rn(dsq[g], add_rn(u, w));
  }
}

template <typename TT>
int pooled_apply(TT *z, const TT *r, const TT *dsq, const float *kern, int H, int W, int half, int b,
                 float *work, cudaStream_t st) {
  const int Hc = (H + b - 1) / b, Wc = (W + b - 1) / b;
  float *uc = work, *wc = work + (size_t)Hc * Wc;
  k_pool<TT><<<mk_grid((int64_t)Hc * Wc, 256, 8), 256, 0, st>>>(r, dsq, uc, H, W, b, Hc, Wc);
  int rc = mk::launch_status("mk_learned_precon_stencil/pool");
  if (!rc) rc = stencil_dispatch<float, true>(wc, uc, nullptr, kern, Hc, Wc, half, st);
  if (rc) return rc;
  k_unpool<TT><<<mk_grid((int64_t)H * W, 256, 8), 256, 0, st>>>(r, dsq, wc, z, H, W, b, Wc);
  return mk::launch_status("mk_learned_precon_stencil/unpool");
}

}  // namespace

extern "C" size_t mk_learned_precon_stencil_work_bytes(int H, int W, int pool) {
  if (H <= 0 || W <= 0 || pool <= 1) return 0;
  const size_t hc = (size_t)(H + pool - 1) / pool, wc = (size_t)(W + pool - 1) / pool;
  return 2 * hc * wc * sizeof(float);
}

extern "C" int mk_learned_precon_stencil(void *z, const void *r, const void *dsq, int H, int W, int half,
                                         const float *kern, int pool, void *work, size_t work_bytes, int dtype,
                                         void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_learned_precon_stencil: bad dtype %d", dtype);
  MK_CHECK_ARG(H > 0 && W > 0, "mk_learned_precon_stencil: bad map shape %d x %d", H, W);
  MK_CHECK_ARG(half >= 0 && half <= ST_MAXHALF, "mk_learned_precon_stencil: half-width %d outside 0..%d", half,
               ST_MAXHALF);
  MK_CHECK_ARG(pool >= 1 && pool <= 64, "mk_learned_precon_stencil: pool factor %d outside 1..64", pool);
  MK_CHECK_ARG(z && r && dsq && kern, "mk_learned_precon_stencil: null pointer");
  MK_CHECK_ARG(z != r, "mk_learned_precon_stencil: z must not alias r (the halo reads neighbours of r)");
  MK_CHECK_ARG(pool == 1 || (work && work_bytes >= mk_learned_precon_stencil_work_bytes(H, W, pool)),
               "mk_learned_precon_stencil: work too small for pool %d (%zu bytes)", pool, work_bytes);
  cudaStream_t st = mk::as_stream(stream);
  if (pool > 1) {
    if (dtype == MK_F64)
      return pooled_apply<double>((double *)z, (const double *)r, (const double *)dsq, kern, H, W, half, pool,
                                  (float *)work, st);
    return pooled_apply<float>((float *)z, (const float *)r, (const float *)dsq, kern, H, W, half, pool,
                               (float *)work, st);
  }
  if (dtype == MK_F64)
    return stencil_dispatch<double>((double *)z, (const double *)r, (const double *)dsq, kern, H, W, half, st);
  return stencil_dispatch<float>((float *)z, (const float *)r, (const float *)dsq, kern, H, W, half, st);
}

extern "C" int mk_conv3x3_fwd(const float *x, const float *w, float *y, int B, int Cin, int Cout, int H,
                              int W, void *stream) {
  int rc = conv_args(B, Cin, Cout, H, W);
  if (rc) return rc;
  MK_CHECK_ARG(x && w && y && x != y, "mk_conv3x3_fwd: bad pointers");
  return conv_launch<false>(x, w, y, B, Cin, Cout, H, W, mk::as_stream(stream), "mk_conv3x3_fwd");
}

extern "C" int mk_conv3x3_adj(const float *y, const float *w, float *x, int B, int Cin, int Cout, int H,
                              int W, void *stream) {
  int rc = conv_args(B, Cin, Cout, H, W);
  if (rc) return rc;
  MK_CHECK_ARG(x && w && y && x != y, "mk_conv3x3_adj: bad pointers");
  return conv_launch<true>(y, w, x, B, Cin, Cout, H, W, mk::as_stream(stream), "mk_conv3x3_adj");
}

extern "C" size_t mk_conv3x3_wgrad_scratch_bytes(int B, int Cin, int Cout, int H, int W) {
  const dim3 g = wgrad_grid(B > 0 ? B : 0, H > 0 ? H : 0, W > 0 ? W : 0);
  return (size_t)g.x * g.y * g.z * (size_t)Cin * Cout * 9 * sizeof(float);
}

extern "C" int mk_conv3x3_wgrad(const float *x, const float *h, float *g, int B, int Cin, int Cout, int H,
                                int W, void *scratch, size_t scratch_bytes, void *stream) {
  int rc = conv_args(B, Cin, Cout, H, W);
  if (rc) return rc;
  MK_CHECK_ARG(x && h && g && scratch, "mk_conv3x3_wgrad: null pointer");
  MK_CHECK_ARG(scratch_bytes >= mk_conv3x3_wgrad_scratch_bytes(B, Cin, Cout, H, W),
               "mk_conv3x3_wgrad: scratch too small");
  static bool attr[64] = {false};
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    MK_CUDA(cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WGRAD_SMEM));
    attr[dev] = true;
  }
  cudaStream_t st = mk::as_stream(stream);
  const dim3 grid = wgrad_grid(B, H, W);
  k_conv_wgrad<<<grid, 256, WGRAD_SMEM, st>>>(x, h, (float *)scratch, Cin, Cout, H, W);
  const int nw = Cin * Cout * 9;
  const int64_t ncta = (int64_t)grid.x * grid.y * grid.z;
  k_wgrad_reduce<<<(nw + 127) / 128, 128, 0, st>>>((const float *)scratch, ncta, nw, g);
  return mk::launch_status("mk_conv3x3_wgrad");
}

extern "C" size_t mk_learned_precon_work_bytes(int H, int W, int nlayer, const int *channels) {
  if (H <= 0 || W <= 0 || nlayer < 1 || !channels) return 0;
  int maxc = 1;
  for (int l = 0; l <= nlayer; l++) maxc = channels[l] > maxc ? channels[l] : maxc;
  return 2 * (size_t)maxc * H * W * sizeof(float);
}

extern "C" int mk_learned_precon_apply(void *z, const void *r, const void *dsq, int H, int W, int nlayer,
                                       const int *channels, const float *const *weights, float *work,
                                       size_t work_bytes, int dtype, void *stream) {
  MK_CHECK_ARG(MK_DTYPE_OK(dtype), "mk_learned_precon_apply: bad dtype %d", dtype);
  MK_CHECK_ARG(nlayer >= 1 && nlayer <= 16 && channels && weights,
               "mk_learned_precon_apply: need 1..16 layers with channels and weights (got %d)", nlayer);
  MK_CHECK_ARG(channels[0] == 1, "mk_learned_precon_apply: the first layer takes 1 channel (got %d)",
               channels[0]);
  for (int l = 1; l <= nlayer; l++) {
    int rc = conv_args(1, channels[l - 1], channels[l], H, W);
    if (rc) return rc;
    MK_CHECK_ARG(weights[l - 1] != nullptr, "mk_learned_precon_apply: layer %d has no weights", l);
  }
  MK_CHECK_ARG(z && r && dsq && work, "mk_learned_precon_apply: null pointer");
  MK_CHECK_ARG(work_bytes >= mk_learned_precon_work_bytes(H, W, nlayer, channels),
               "mk_learned_precon_apply: work too small (%zu bytes)", work_bytes);
  int maxc = 1;
  for (int l = 0; l <= nlayer; l++) maxc = channels[l] > maxc ? channels[l] : maxc;
  cudaStream_t st = mk::as_stream(stream);
  if (dtype == MK_F64)
    return precon_apply<double>((double *)z, (const double *)r, (const double *)dsq, H, W, nlayer, channels,
                                weights, work, maxc, st);
  return precon_apply<float>((float *)z, (const float *)r, (const float *)dsq, H, W, nlayer, channels, weights,
                             work, maxc, st);
}
