// 3x3 convolutions for the learned SPD map-space preconditioner
//   M = D^-1/2 (I + K^T K) D^-1/2,  K = L4 L3 L2 L1 (linear 3x3 convolutions)
// applied to map-sized PCG residuals.  Three kernels cover inference and
// training:
//   conv_fwd : Y[b,co,p]  = sum_ci sum_d W[co,ci,d] X[b,ci,p+d]       (L x)
//   conv_adj : X[b,ci,q]  = sum_co sum_d W[co,ci,d] Y[b,co,q-d]       (L^T y)
//   conv_wgrad: G[co,ci,d] = sum_b sum_p H[b,co,p] X[b,ci,p+d]
// with zero padding (pixels outside the map are 0).  Layout: [B][C][H][W],
// FP32, at most 16 channels.  A CTA owns a 16x16 pixel tile of one map and
// stages the input tile plus a 1-pixel halo for every channel in shared
// memory; the weights (<= 16*16*9 floats) sit in shared memory and are read
// as warp-wide broadcasts.  conv_wgrad writes one partial per CTA and a
// second kernel sums the partials in a fixed order (reproducible gradients).
#include "mk_common.cuh"

namespace {

constexpr int CMAX = 16;
constexpr int T = 16;            // tile edge
constexpr int TH = T + 2;        // with halo
constexpr int NW = CMAX * CMAX * 9;

__device__ __forceinline__ float ld_pad(const float *__restrict__ x, int H, int W, int y, int xx) {
  return (y >= 0 && y < H && xx >= 0 && xx < W) ? x[(int64_t)y * W + xx] : 0.f;
}

__global__ void __launch_bounds__(256) k_conv_fwd(const float *__restrict__ X, const float *__restrict__ Wt,
                                                  float *__restrict__ Y, int Cin, int Cout, int H, int W) {
  __shared__ float sx[CMAX][TH][TH];
  __shared__ float sw[NW];
  const int b = blockIdx.z;
  const int y0 = blockIdx.y * T, x0 = blockIdx.x * T;
  const int tid = threadIdx.x;
  for (int i = tid; i < Cout * Cin * 9; i += 256) sw[i] = Wt[i];
  const float *xb = X + (int64_t)b * Cin * H * W;
  for (int i = tid; i < Cin * TH * TH; i += 256) {
    int c = i / (TH * TH), r = (i / TH) % TH, q = i % TH;
    sx[c][r][q] = ld_pad(xb + (int64_t)c * H * W, H, W, y0 + r - 1, x0 + q - 1);
  }
  __syncthreads();
  const int ty = tid / T, tx = tid % T;
  float acc[CMAX];
#pragma unroll
  for (int co = 0; co < CMAX; co++) acc[co] = 0.f;
  for (int ci = 0; ci < Cin; ci++) {
#pragma unroll
    for (int d = 0; d < 9; d++) {
      const float v = sx[ci][ty + d / 3][tx + d % 3];
#pragma unroll
      for (int co = 0; co < CMAX; co++)
        if (co < Cout) acc[co] = fmaf(sw[(co * Cin + ci) * 9 + d], v, acc[co]);
    }
  }
  const int yy = y0 + ty, xx = x0 + tx;
  if (yy < H && xx < W) {
    float *yb = Y + (int64_t)b * Cout * H * W + (int64_t)yy * W + xx;
#pragma unroll
    for (int co = 0; co < CMAX; co++)
      if (co < Cout) yb[(int64_t)co * H * W] = acc[co];
  }
}

// adjoint: the tap d of output pixel p reads input pixel p+d, so input pixel
// q receives from output pixels q-d.
__global__ void __launch_bounds__(256) k_conv_adj(const float *__restrict__ Yin, const float *__restrict__ Wt,
                                                  float *__restrict__ Xout, int Cin, int Cout, int H, int W) {
  __shared__ float sy[CMAX][TH][TH];
  __shared__ float sw[NW];
  const int b = blockIdx.z;
  const int y0 = blockIdx.y * T, x0 = blockIdx.x * T;
  const int tid = threadIdx.x;
  for (int i = tid; i < Cout * Cin * 9; i += 256) sw[i] = Wt[i];
  const float *yb = Yin + (int64_t)b * Cout * H * W;
  for (int i = tid; i < Cout * TH * TH; i += 256) {
    int c = i / (TH * TH), r = (i / TH) % TH, q = i % TH;
    sy[c][r][q] = ld_pad(yb + (int64_t)c * H * W, H, W, y0 + r - 1, x0 + q - 1);
  }
  __syncthreads();
  const int ty = tid / T, tx = tid % T;
  float acc[CMAX];
#pragma unroll
  for (int ci = 0; ci < CMAX; ci++) acc[ci] = 0.f;
  for (int co = 0; co < Cout; co++) {
#pragma unroll
    for (int d = 0; d < 9; d++) {
      // q - d with d = (dy-1, dx-1): tile index (ty + 1 - (dy-1), tx + 1 - (dx-1))
      const float v = sy[co][ty + 2 - d / 3][tx + 2 - d % 3];
#pragma unroll
      for (int ci = 0; ci < CMAX; ci++)
        if (ci < Cin) acc[ci] = fmaf(sw[(co * Cin + ci) * 9 + d], v, acc[ci]);
    }
  }
  const int yy = y0 + ty, xx = x0 + tx;
  if (yy < H && xx < W) {
    float *xb = Xout + (int64_t)b * Cin * H * W + (int64_t)yy * W + xx;
#pragma unroll
    for (int ci = 0; ci < CMAX; ci++)
      if (ci < Cin) xb[(int64_t)ci * H * W] = acc[ci];
  }
}

// one partial gradient per CTA: part[cta][co][ci][d]
__global__ void __launch_bounds__(256) k_conv_wgrad(const float *__restrict__ X, const float *__restrict__ Hg,
                                                    float *__restrict__ part, int Cin, int Cout, int H, int W) {
  __shared__ float sx[CMAX][TH][TH];
  __shared__ float sh[CMAX][T][T];
  const int b = blockIdx.z;
  const int y0 = blockIdx.y * T, x0 = blockIdx.x * T;
  const int tid = threadIdx.x;
  const float *xb = X + (int64_t)b * Cin * H * W;
  const float *hb = Hg + (int64_t)b * Cout * H * W;
  for (int i = tid; i < Cin * TH * TH; i += 256) {
    int c = i / (TH * TH), r = (i / TH) % TH, q = i % TH;
    sx[c][r][q] = ld_pad(xb + (int64_t)c * H * W, H, W, y0 + r - 1, x0 + q - 1);
  }
  for (int i = tid; i < Cout * T * T; i += 256) {
    int c = i / (T * T), r = (i / T) % T, q = i % T;
    int yy = y0 + r, xx = x0 + q;
    sh[c][r][q] = (yy < H && xx < W) ? hb[(int64_t)c * H * W + (int64_t)yy * W + xx] : 0.f;
  }
  __syncthreads();
  const int nw = Cout * Cin * 9;
  const int64_t cta = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  for (int w = tid; w < nw; w += 256) {
    const int co = w / (Cin * 9), ci = (w / 9) % Cin, d = w % 9;
    const int dy = d / 3, dx = d % 3;
    float acc = 0.f;
    for (int r = 0; r < T; r++)
#pragma unroll
      for (int q = 0; q < T; q++) acc = fmaf(sh[co][r][q], sx[ci][r + dy][q + dx], acc);
    part[cta * nw + w] = acc;
  }
}

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

dim3 conv_grid(int B, int H, int W) { return dim3((W + T - 1) / T, (H + T - 1) / T, B); }

}  // namespace

extern "C" int mk_conv3x3_fwd(const float *x, const float *w, float *y, int B, int Cin, int Cout, int H,
                              int W, void *stream) {
  int rc = conv_args(B, Cin, Cout, H, W);
  if (rc) return rc;
  MK_CHECK_ARG(x && w && y && x != y, "mk_conv3x3_fwd: bad pointers");
  k_conv_fwd<<<conv_grid(B, H, W), 256, 0, mk::as_stream(stream)>>>(x, w, y, Cin, Cout, H, W);
  return mk::launch_status("mk_conv3x3_fwd");
}

extern "C" int mk_conv3x3_adj(const float *y, const float *w, float *x, int B, int Cin, int Cout, int H,
                              int W, void *stream) {
  int rc = conv_args(B, Cin, Cout, H, W);
  if (rc) return rc;
  MK_CHECK_ARG(x && w && y && x != y, "mk_conv3x3_adj: bad pointers");
  k_conv_adj<<<conv_grid(B, H, W), 256, 0, mk::as_stream(stream)>>>(y, w, x, Cin, Cout, H, W);
  return mk::launch_status("mk_conv3x3_adj");
}

extern "C" size_t mk_conv3x3_wgrad_scratch_bytes(int B, int Cin, int Cout, int H, int W) {
  size_t ncta = (size_t)((W + T - 1) / T) * ((H + T - 1) / T) * (size_t)(B > 0 ? B : 0);
  return ncta * (size_t)Cin * Cout * 9 * sizeof(float);
}

extern "C" int mk_conv3x3_wgrad(const float *x, const float *h, float *g, int B, int Cin, int Cout, int H,
                                int W, void *scratch, size_t scratch_bytes, void *stream) {
  int rc = conv_args(B, Cin, Cout, H, W);
  if (rc) return rc;
  MK_CHECK_ARG(x && h && g && scratch, "mk_conv3x3_wgrad: null pointer");
  MK_CHECK_ARG(scratch_bytes >= mk_conv3x3_wgrad_scratch_bytes(B, Cin, Cout, H, W),
               "mk_conv3x3_wgrad: scratch too small");
  cudaStream_t st = mk::as_stream(stream);
  dim3 grid = conv_grid(B, H, W);
  k_conv_wgrad<<<grid, 256, 0, st>>>(x, h, (float *)scratch, Cin, Cout, H, W);
  int nw = Cin * Cout * 9;
  int64_t ncta = (int64_t)grid.x * grid.y * grid.z;
  k_wgrad_reduce<<<(nw + 127) / 128, 128, 0, st>>>((const float *)scratch, ncta, nw, g);
  return mk::launch_status("mk_conv3x3_wgrad");
}
