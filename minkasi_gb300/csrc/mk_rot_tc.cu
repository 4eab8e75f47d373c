// Detector rotation R = A . X on the 5th-generation tensor cores
// (tcgen05.mma kind::tf32), FP32 in / FP32 out, 3xTF32 split precision:
//   A = Ah + Al, X = Xh + Xl (h = round-to-TF32, l = remainder, also TF32)
//   R ~= Xh.Ah + Xl.Ah + Xh.Al   accumulated in FP32 in tensor memory.
// The dropped Xl.Al term is ~2^-22 relative, so the result carries FP32-level
// accuracy (the apply_noise rotations np.dot(v, dat), np.dot(vT, .) of
// minkasi/mapmaking/noise.py:704,709).
//
// Tile mapping (all operands K-major, 128-byte swizzle):
//   D^T (128 samples x ndet) = X^T (128 samples x K=ndet) . A^T (K x N=ndet)
//   MMA A-operand: the X^T tile.  Each thread owns one sample row; it loads
//     its 32 detector values of a K-chunk (coalesced across the warp: 32
//     consecutive samples of one detector row), splits them, and writes the
//     hi and lo rows (128 B each) into shared memory.
//   MMA B-operand: rows j = output detector, K contiguous = A[j][k0..k0+31],
//     i.e. A row-major.  Its hi/lo split is built once per call by k_bprep
//     in exactly the shared-memory image and bulk-copied (cp.async.bulk)
//     per K-chunk, completing on an mbarrier.
//   Accumulator: 128 TMEM lanes (= samples) x ndet columns (= detectors).
//   Epilogue: each warp reads its 32 lanes with tcgen05.ld 32x32b and
//     stores, per detector column, 32 consecutive samples (128 B, coalesced).
// Pipeline: 2 shared-memory stages; the MMAs of chunk g run while the
// threads split chunk g+1.  One elected thread issues the MMAs and the bulk
// copies.  Every mbarrier wait is bounded: on timeout the CTA records an
// error code, waits (bounded) for its outstanding MMAs, frees its tensor
// memory and returns.
#include <cstdlib>

#include "mk_async.cuh"
#include "mk_common.cuh"
#include "mk_rot.cuh"

namespace {

using mk::bulk_g2s;
using mk::mbar_expect_tx;
using mk::mbar_init;
using mk::mbar_wait;
using mk::smem_u32;

constexpr int TILE_M = 128;      // samples per tile (MMA M)
constexpr int KC = 32;           // K per chunk: one 128-byte swizzle row of tf32
constexpr int NSTAGE = 2;
constexpr int NTHREADS = 128;

__device__ __forceinline__ float tf32_round(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

// byte offset of element (row, k) in a K-major, 128B-swizzled tile whose
// rows hold 32 fp32 (one swizzle row each); 8-row groups are 1024 B apart.
__host__ __device__ __forceinline__ uint32_t sw128_off(uint32_t row, uint32_t k) {
  return (row >> 3) * 1024u + (row & 7u) * 128u + ((((k >> 2) ^ (row & 7u)) & 7u) << 4) + (k & 3u) * 4u;
}

// shared-memory matrix descriptor: K-major, SWIZZLE_128B, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);          // start address
  d |= (uint64_t)1 << 16;                              // leading byte offset (unused for SW128 K-major)
  d |= (uint64_t)(1024u >> 4) << 32;                   // stride byte offset
  d |= (uint64_t)1 << 46;                              // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                              // swizzle: 128B
  return d;
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
        "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
        "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// B-operand image in global memory: for each K-chunk c, the hi tile then the
// lo tile, each ndet rows x 32 k in the swizzled layout above.
__global__ void k_bprep(const float *__restrict__ A, int ndet, char *__restrict__ img) {
  const int nchunk = ndet / KC;
  const size_t tile = (size_t)ndet * 128;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < ndet * ndet; idx += gridDim.x * blockDim.x) {
    int j = idx / ndet, k = idx % ndet;
    int c = k / KC, kk = k % KC;
    float a = A[(size_t)j * ndet + k];
    float h = tf32_round(a);
    float l = tf32_round(a - h);
    char *base = img + (size_t)c * 2 * tile;
    *(float *)(base + sw128_off(j, kk)) = h;
    *(float *)(base + tile + sw128_off(j, kk)) = l;
  }
  (void)nchunk;
}

// shared memory: [stage][Ahi 16KB | Alo 16KB | Bhi ndet*128 | Blo ndet*128], 1024-aligned
// Raw X chunks (32 detectors x 128 samples, 16 KB) are fetched RSTAGE chunks
// ahead with 4-byte cp.async into a ring in shared memory.  Each thread
// copies exactly the 32 values of its own sample row, so after its own
// cp.async.wait_group it can read them back without a CTA barrier.
constexpr int RSTAGE = 2;

__device__ __forceinline__ void cp_async4(float *dst, const float *src, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// queue the copy of chunk q (tile, c) of this CTA into raw slot q % RSTAGE;
// always commits one group so that group counting stays uniform
__device__ __forceinline__ void prefetch_chunk(const float *__restrict__ X, int64_t ldx, int64_t xs, int64_t ncol,
                                               int nchunk, int64_t ntile, uint32_t q, float *raw,
                                               int tid) {
  const int64_t tile = blockIdx.x + (int64_t)(q / nchunk) * gridDim.x;
  const int c = (int)(q % nchunk);
  if (tile < ntile) {
    const int64_t my = tile * TILE_M + tid;
    const bool ok = my < ncol;
    const float *src = X + (int64_t)(c * KC) * ldx + (ok ? my : 0) * xs;
    float *dst = raw + (size_t)(q % RSTAGE) * KC * TILE_M + tid;
#pragma unroll
    for (int kk = 0; kk < KC; kk++) cp_async4(dst + kk * TILE_M, src + (int64_t)kk * ldx, ok);
  }
  cp_async_commit();
}

__global__ void __launch_bounds__(NTHREADS, 1)
    k_rot_tc(const float *__restrict__ X, int64_t ldx, float *__restrict__ R, int64_t ldr, int ndet,
             int64_t ncol, const char *__restrict__ bimg, int *__restrict__ err, int64_t mirror_n,
             int64_t xs, int halve_ends) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t a_bytes = TILE_M * 128;          // 16 KB
  const uint32_t b_bytes = (uint32_t)ndet * 128;  // per hi or lo tile
  const uint32_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
  float *raw = (float *)(smem + NSTAGE * stage_bytes);
  __shared__ uint64_t bar_b[NSTAGE], bar_mma[NSTAGE];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh;

  const int tid = threadIdx.x, warp = tid >> 5;
  const int nchunk = ndet / KC;
  const uint32_t ncols = ndet < 32 ? 32u : (uint32_t)ndet;  // power of two by construction
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(ndet >> 3) << 17) |
                         ((uint32_t)(TILE_M >> 4) << 24);

  if (tid == 0) {
    for (int s = 0; s < NSTAGE; s++) {
      mbar_init(&bar_b[s], 1);
      mbar_init(&bar_mma[s], 1);
    }
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base_sh;

  // Control flow is CTA-uniform: only thread 0 waits on mbarriers; the
  // outcome reaches the other threads through abort_sh and __syncthreads.
  const int64_t ntile = (ncol + TILE_M - 1) / TILE_M;
  for (uint32_t q = 0; q < (uint32_t)RSTAGE; q++) prefetch_chunk(X, ldx, xs, ncol, nchunk, ntile, q, raw, tid);
  uint32_t g = 0;  // chunks issued by this CTA so far
  for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int64_t n0 = tile * TILE_M;
    const int64_t my = n0 + tid;
    // DCT-I endpoint halving folded into the load (noise.py:710-711)
    const float hscale = (halve_ends && (my == 0 || my == ncol - 1)) ? 0.5f : 1.0f;
    for (int c = 0; c < nchunk; c++, g++) {
      const uint32_t s = g % NSTAGE, use = g / NSTAGE;
      unsigned char *st = smem + s * stage_bytes;
      // this thread's sample row: 32 detectors of chunk c from the raw ring,
      // split into hi / lo; then queue the chunk RSTAGE ahead into that slot
      float h[KC], l[KC];
      cp_async_wait<RSTAGE - 1>();
      const float *rw = raw + (size_t)(g % RSTAGE) * KC * TILE_M + tid;
#pragma unroll
      for (int kk = 0; kk < KC; kk++) {
        float x = rw[kk * TILE_M] * hscale;
        h[kk] = tf32_round(x);
        l[kk] = tf32_round(x - h[kk]);
      }
      prefetch_chunk(X, ldx, xs, ncol, nchunk, ntile, g + RSTAGE, raw, tid);
      if (tid == 0) {
        // stage s is free once the MMAs of chunk g-2 have completed
        if (g >= NSTAGE && !mbar_wait(&bar_mma[s], (use - 1) & 1)) {
          abort_sh = 1;
        } else {
          mbar_expect_tx(&bar_b[s], 2 * b_bytes);
          bulk_g2s(st + 2 * a_bytes, bimg + (size_t)c * 2 * b_bytes, 2 * b_bytes, &bar_b[s]);
        }
      }
      __syncthreads();
      if (abort_sh) break;
      unsigned char *ah = st, *al = st + a_bytes;
#pragma unroll
      for (int q = 0; q < KC / 4; q++) {
        uint32_t off = sw128_off(tid, 4 * q);
        *(float4 *)(ah + off) = make_float4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
        *(float4 *)(al + off) = make_float4(l[4 * q], l[4 * q + 1], l[4 * q + 2], l[4 * q + 3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        if (!mbar_wait(&bar_b[s], use & 1)) {
          abort_sh = 1;  // seen by everyone at the next __syncthreads
        } else {
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t sa_h = smem_u32(ah), sa_l = smem_u32(al);
          const uint32_t sb_h = smem_u32(st + 2 * a_bytes), sb_l = sb_h + b_bytes;
#pragma unroll
          for (int k8 = 0; k8 < KC / 8; k8++) {
            const uint32_t ko = k8 * 32;  // 8 tf32 = 32 bytes along K
            const uint32_t acc0 = (c == 0 && k8 == 0) ? 0u : 1u;
            mma_tf32(tmem, sdesc(sa_h + ko), sdesc(sb_h + ko), idesc, acc0);
            mma_tf32(tmem, sdesc(sa_l + ko), sdesc(sb_h + ko), idesc, 1u);
            mma_tf32(tmem, sdesc(sa_h + ko), sdesc(sb_l + ko), idesc, 1u);
          }
          mma_commit(&bar_mma[s]);
        }
      }
    }
    // epilogue: wait for the tile's last chunk, TMEM -> registers -> R
    if (tid == 0 && !abort_sh) {
      const uint32_t sl = (g - 1) % NSTAGE, ul = (g - 1) / NSTAGE;
      if (!mbar_wait(&bar_mma[sl], ul & 1)) abort_sh = 1;
    }
    __syncthreads();
    if (abort_sh) break;
    asm volatile("tcgen05.fence::after_thread_sync;");
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    for (int c0 = 0; c0 < ndet; c0 += 32) {
      float v[32];
      tmem_ld32(tmem + lane_base + (uint32_t)c0, v);
      if (my < ncol) {
#pragma unroll
        for (int j = 0; j < 32; j++) __stcs(R + (int64_t)(c0 + j) * ldr + my, v[j]);
        // even extension for the DCT-I that follows: R[., mirror_n - my] = R[., my]
        if (mirror_n > 0 && my >= 1 && my <= ncol - 2) {
#pragma unroll
          for (int j = 0; j < 32; j++) __stcs(R + (int64_t)(c0 + j) * ldr + (mirror_n - my), v[j]);
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
  }
  cp_async_wait<0>();  // no copy into this CTA's shared memory outlives it
  if (abort_sh && tid == 0) {
    atomicExch(err, 1);
    // bounded drain of MMAs possibly still in flight before freeing tensor memory
    for (uint32_t q = (g > NSTAGE ? g - NSTAGE : 0); q < g; q++)
      (void)mbar_wait(&bar_mma[q % NSTAGE], (q / NSTAGE) & 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// ---- warp-specialised version ---------------------------------------------
// The same tiles, products and operand images, with the roles split so that
// no CTA-wide barrier sits in the main loop:
//   warps 0-3 (split): thread t owns sample row t of every tile; it splits its
//     32 values of a K-chunk into hi / lo and writes them into the chunk's
//     A stage, then arrives on full_a[stage];
//   warp 4, lane 0 (MMA): bulk-copies the chunk's B image into the stage
//     (full_b[stage]), waits for both halves, issues the 12 MMAs and commits
//     them to mma_done[stage] (which frees the stage for chunk g + 2); after
//     a tile's last chunk it commits to acc_full[buffer];
//   warps 5-8 (epilogue): tensor memory holds two accumulators (2 x ndet
//     columns), so while the MMAs of tile i + 1 run, these warps read tile i
//     (warp w reads TMEM lanes 32 (w % 4) ..) and store it, then arrive on
//     acc_empty[buffer].
// Every wait is bounded and also polls the CTA's abort flag, so a timeout in
// one role ends all of them; the MMA thread then drains its outstanding
// MMAs (bounded) before the tensor memory is freed.
constexpr int WS_SPLIT = 4, WS_EPI = 4;
constexpr int WS_THREADS = (WS_SPLIT + 1 + WS_EPI) * 32;

__device__ __forceinline__ bool ws_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag) {
  for (uint32_t i = 0; i < mk::SPIN_LIMIT; i++) {
    if (mk::mbar_try_wait(bar, parity)) return true;
    if ((i & 31u) == 31u && *abort_flag) return false;
  }
  *abort_flag = 1;
  return false;
}

// The job (TOD) that owns tile t of the launch; jobs are sorted by tile0 and
// each role walks its tiles in increasing order, so the cursor only moves on.
__device__ __forceinline__ int job_at(const mk::RotJob *jobs, int njobs, int64_t t, int cur) {
  while (cur + 1 < njobs && jobs[cur + 1].tile0 <= t) cur++;
  return cur;
}

// queue the copy of chunk q of this CTA (tile blockIdx.x + (q / nchunk) *
// gridDim.x, K-chunk q % nchunk) into raw slot q % RSTAGE; always commits one
// group so that group counting stays uniform
__device__ __forceinline__ void prefetch_job(const mk::RotJob *jobs, int njobs, int &pcur, int64_t xs, int nchunk,
                                             int64_t ntile, uint32_t q, float *raw, int tid) {
  const int64_t tile = blockIdx.x + (int64_t)(q / nchunk) * gridDim.x;
  const int c = (int)(q % nchunk);
  if (tile < ntile) {
    pcur = job_at(jobs, njobs, tile, pcur);
    const mk::RotJob &J = jobs[pcur];
    const int64_t my = (tile - J.tile0) * TILE_M + tid;
    const bool ok = my < J.ncol;
    const float *src = J.X + (int64_t)(c * KC) * J.ldx + (ok ? my : 0) * xs;
    float *dst = raw + (size_t)(q % RSTAGE) * KC * TILE_M + tid;
#pragma unroll
    for (int kk = 0; kk < KC; kk++) cp_async4(dst + kk * TILE_M, src + (int64_t)kk * J.ldx, ok);
  }
  cp_async_commit();
}

// `jobs` (device memory, sorted by tile0) lists the TODs of a grouped launch,
// all with ndet detectors; for one TOD it is null and `j0` is that TOD.
// mirror_n, xs and halve_ends apply to single-TOD launches (0, 1, 0 in groups).
__global__ void __launch_bounds__(WS_THREADS, 1)
    k_rot_tc_ws(const mk::RotJob *__restrict__ jobs_in, int njobs, const mk::RotJob j0, int64_t ntile, int ndet,
                int *__restrict__ err, int64_t mirror_n, int64_t xs, int halve_ends) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const uint32_t a_bytes = TILE_M * 128;
  const uint32_t b_bytes = (uint32_t)ndet * 128;
  const uint32_t stage_bytes = 2 * a_bytes + 2 * b_bytes;
  float *raw = (float *)(smem + NSTAGE * stage_bytes);
  __shared__ uint64_t full_a[NSTAGE], full_b[NSTAGE], mma_done[NSTAGE], acc_full[2], acc_empty[2];
  __shared__ uint32_t tmem_base_sh;
  __shared__ int abort_sh;
  volatile int *abort_flag = &abort_sh;
  const mk::RotJob *jobs = jobs_in ? jobs_in : &j0;
  if (!jobs_in) njobs = 1;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nchunk = ndet / KC;
  const uint32_t ncols = 2u * (ndet < 32 ? 32u : (uint32_t)ndet);  // two accumulators, a power of two
  const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(ndet >> 3) << 17) |
                         ((uint32_t)(TILE_M >> 4) << 24);
  if (tid == 0) {
    for (int s = 0; s < NSTAGE; s++) {
      mbar_init(&full_a[s], WS_SPLIT * 32);
      mbar_init(&full_b[s], 1);
      mbar_init(&mma_done[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], WS_EPI * 32);
    }
    abort_sh = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&tmem_base_sh)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base_sh;
  uint32_t g_issued = 0;  // MMA thread: chunks whose MMAs were committed

  if (warp < WS_SPLIT) {
    // ---- split role ----
    int pcur = 0, cur = 0;
    for (uint32_t q = 0; q < (uint32_t)RSTAGE; q++) prefetch_job(jobs, njobs, pcur, xs, nchunk, ntile, q, raw, tid);
    uint32_t g = 0;
    for (int64_t tile = blockIdx.x; tile < ntile && !*abort_flag; tile += gridDim.x) {
      cur = job_at(jobs, njobs, tile, cur);
      const int64_t my = (tile - jobs[cur].tile0) * TILE_M + tid, ncol = jobs[cur].ncol;
      const float hscale = (halve_ends && (my == 0 || my == ncol - 1)) ? 0.5f : 1.0f;
      for (int c = 0; c < nchunk; c++, g++) {
        const uint32_t s = g % NSTAGE, use = g / NSTAGE;
        float h[KC], l[KC];
        cp_async_wait<RSTAGE - 1>();
        const float *rw = raw + (size_t)(g % RSTAGE) * KC * TILE_M + tid;
#pragma unroll
        for (int kk = 0; kk < KC; kk++) {
          const float x = rw[kk * TILE_M] * hscale;
          h[kk] = tf32_round(x);
          l[kk] = tf32_round(x - h[kk]);
        }
        prefetch_job(jobs, njobs, pcur, xs, nchunk, ntile, g + RSTAGE, raw, tid);
        if (g >= NSTAGE && !ws_wait(&mma_done[s], (use - 1) & 1, abort_flag)) break;
        unsigned char *ah = smem + s * stage_bytes, *al = ah + a_bytes;
#pragma unroll
        for (int q = 0; q < KC / 4; q++) {
          const uint32_t off = sw128_off(tid, 4 * q);
          *(float4 *)(ah + off) = make_float4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
          *(float4 *)(al + off) = make_float4(l[4 * q], l[4 * q + 1], l[4 * q + 2], l[4 * q + 3]);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mk::mbar_arrive(&full_a[s]);
      }
    }
    cp_async_wait<0>();  // no copy into this CTA's shared memory outlives it
  } else if (warp == WS_SPLIT) {
    // ---- MMA role (one thread) ----
    if (lane == 0) {
      uint32_t g = 0;
      int64_t it = 0;
      int cur = 0;
      for (int64_t tile = blockIdx.x; tile < ntile && !*abort_flag; tile += gridDim.x, it++) {
        cur = job_at(jobs, njobs, tile, cur);
        const char *bimg = jobs[cur].bimg;
        const uint32_t ab = (uint32_t)(it & 1), au = (uint32_t)(it >> 1);
        if (it >= 2 && !ws_wait(&acc_empty[ab], (au - 1) & 1, abort_flag)) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t dacc = tmem + ab * (ncols / 2);
        bool ok = true;
        for (int c = 0; c < nchunk; c++, g++) {
          const uint32_t s = g % NSTAGE, use = g / NSTAGE;
          unsigned char *st = smem + s * stage_bytes;
          if (g >= NSTAGE && !ws_wait(&mma_done[s], (use - 1) & 1, abort_flag)) {
            ok = false;
            break;
          }
          mbar_expect_tx(&full_b[s], 2 * b_bytes);
          bulk_g2s(st + 2 * a_bytes, bimg + (size_t)c * 2 * b_bytes, 2 * b_bytes, &full_b[s]);
          if (!ws_wait(&full_b[s], use & 1, abort_flag) || !ws_wait(&full_a[s], use & 1, abort_flag)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t sa_h = smem_u32(st), sa_l = sa_h + a_bytes;
          const uint32_t sb_h = smem_u32(st + 2 * a_bytes), sb_l = sb_h + b_bytes;
#pragma unroll
          for (int k8 = 0; k8 < KC / 8; k8++) {
            const uint32_t ko = k8 * 32;
            const uint32_t acc0 = (c == 0 && k8 == 0) ? 0u : 1u;
            mma_tf32(dacc, sdesc(sa_h + ko), sdesc(sb_h + ko), idesc, acc0);
            mma_tf32(dacc, sdesc(sa_l + ko), sdesc(sb_h + ko), idesc, 1u);
            mma_tf32(dacc, sdesc(sa_h + ko), sdesc(sb_l + ko), idesc, 1u);
          }
          mma_commit(&mma_done[s]);
          g_issued = g + 1;
        }
        if (!ok) break;
        mma_commit(&acc_full[ab]);
      }
    }
  } else {
    // ---- epilogue role ----
    const int q = warp & 3;  // TMEM lane quarter this warp may access
    const int row = 32 * q + lane;
    int64_t it = 0;
    int cur = 0;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x, it++) {
      cur = job_at(jobs, njobs, tile, cur);
      const uint32_t ab = (uint32_t)(it & 1), au = (uint32_t)(it >> 1);
      // every lane waits; the warp goes on only if all of them saw the
      // phase complete (tcgen05.ld below needs the whole warp converged)
      const bool okw = ws_wait(&acc_full[ab], au & 1, abort_flag);
      if (!__all_sync(0xffffffffu, okw)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const mk::RotJob &J = jobs[cur];
      const int64_t my = (tile - J.tile0) * TILE_M + row, ncol = J.ncol, ldr = J.ldr;
      float *R = J.R;
      const uint32_t base = tmem + ((uint32_t)(32 * q) << 16) + ab * (ncols / 2);
      for (int c0 = 0; c0 < ndet; c0 += 32) {
        float v[32];
        tmem_ld32(base + (uint32_t)c0, v);
        if (my < ncol) {
#pragma unroll
          for (int j = 0; j < 32; j++) __stcs(R + (int64_t)(c0 + j) * ldr + my, v[j]);
          if (mirror_n > 0 && my >= 1 && my <= ncol - 2) {
#pragma unroll
            for (int j = 0; j < 32; j++) __stcs(R + (int64_t)(c0 + j) * ldr + (mirror_n - my), v[j]);
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      mk::mbar_arrive(&acc_empty[ab]);
    }
  }
  __syncthreads();
  if (*abort_flag && tid == WS_SPLIT * 32) {
    atomicExch(err, 1);
    // bounded drain of the MMAs this thread issued before freeing tensor memory
    for (uint32_t g = (g_issued > NSTAGE ? g_issued - NSTAGE : 0); g < g_issued; g++)
      (void)mbar_wait(&mma_done[g % NSTAGE], (g / NSTAGE) & 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

size_t ws_smem_bytes(int nd) {
  const size_t stage = 2 * (size_t)TILE_M * 128 + 2 * (size_t)nd * 128;
  return NSTAGE * stage + (size_t)RSTAGE * KC * TILE_M * sizeof(float) + 1024;
}

int ws_prepare(size_t smem) {
  static int attr_ws[64] = {0};
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && attr_ws[dev] < (int)smem) {
    MK_CUDA(cudaFuncSetAttribute(k_rot_tc_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_ws[dev] = (int)smem;
  }
  return MK_OK;
}

}  // namespace

namespace mk {

bool rot_tc_supported(int64_t nrow) {
  return nrow == 32 || nrow == 64 || nrow == 128 || nrow == 256;
}

size_t rot_tc_bimg_bytes(int64_t nrow) { return (size_t)nrow * (size_t)nrow * 8; }

int rot_tc_f32(const float *A, const float *X, int64_t ldx, float *R, int64_t ldr, int64_t nrow,
               int64_t ncol, void *bimg, int *err, cudaStream_t st, int64_t mirror_n, int64_t x_stride,
               int halve_ends) {
  MK_CHECK_ARG(rot_tc_supported(nrow), "tensor-core rotation supports ndet in {32,64,128,256}, got %lld",
               (long long)nrow);
  MK_CHECK_ARG(bimg && err && ((uintptr_t)bimg % 16) == 0, "tensor-core rotation: bad scratch");
  MK_CHECK_ARG(mirror_n == 0 || (mirror_n == 2 * (ncol - 1) && ldr >= mirror_n),
               "tensor-core rotation: bad mirror extent");
  MK_CHECK_ARG(x_stride == 1 || x_stride == 2, "tensor-core rotation: element stride must be 1 or 2");
  if (ncol <= 0) return MK_OK;
  const int nd = (int)nrow;
  k_bprep<<<(nd * nd + 255) / 256, 256, 0, st>>>(A, nd, (char *)bimg);
  const size_t stage = 2 * (size_t)TILE_M * 128 + 2 * (size_t)nd * 128;
  const size_t smem = NSTAGE * stage + (size_t)RSTAGE * KC * TILE_M * sizeof(float) + 1024;
  static int attr_set[64] = {0};
  int dev = 0;
  MK_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && attr_set[dev] < (int)smem) {
    MK_CUDA(cudaFuncSetAttribute(k_rot_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set[dev] = (int)smem;
  }
  int64_t ntile = (ncol + TILE_M - 1) / TILE_M;
  // one TOD: the single-role kernel, measured 10 % faster than the
  // warp-specialised one on a 256 x 130,978 TOD (both wait on the loads of
  // X: two 16 KB chunks in flight per SM); MINKASI_GB300_ROT_TC_WS=1 selects
  // the warp-specialised kernel, which the grouped (many-TOD) launch uses
  static const bool ws = [] {
    const char *e = getenv("MINKASI_GB300_ROT_TC_WS");
    return e && e[0] == '1';
  }();
  if (ws) {
    const size_t wsmem = ws_smem_bytes(nd);
    int rc = ws_prepare(wsmem);
    if (rc) return rc;
    RotJob j0{X, R, (const char *)bimg, ldx, ldr, ncol, 0};
    // one CTA per SM: its two accumulators take up to all 512 TMEM columns
    int64_t grid = (int64_t)sm_count();
    if (grid > ntile) grid = ntile;
    k_rot_tc_ws<<<(unsigned)grid, WS_THREADS, wsmem, st>>>(nullptr, 1, j0, ntile, nd, err, mirror_n, x_stride,
                                                           halve_ends);
    return launch_status("rot_tc_f32");
  }
  int per_sm = (int)(220 * 1024 / smem);
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 2) per_sm = 2;  // tensor memory: <= 2 x 256 columns per SM
  int64_t grid = (int64_t)sm_count() * per_sm;
  if (grid > ntile) grid = ntile;
  k_rot_tc<<<(unsigned)grid, NTHREADS, smem, st>>>(X, ldx, R, ldr, nd, ncol, (const char *)bimg, err,
                                                   mirror_n, x_stride, halve_ends);
  return launch_status("rot_tc_f32");
}

}  // namespace mk

namespace mk {

int rot_tc_bprep(const float *A, int64_t nrow, void *bimg, cudaStream_t st) {
  MK_CHECK_ARG(rot_tc_supported(nrow), "tensor-core rotation supports ndet in {32,64,128,256}, got %lld",
               (long long)nrow);
  MK_CHECK_ARG(A && bimg && ((uintptr_t)bimg % 16) == 0, "tensor-core rotation: bad operand image");
  const int nd = (int)nrow;
  k_bprep<<<(nd * nd + 255) / 256, 256, 0, st>>>(A, nd, (char *)bimg);
  return launch_status("rot_tc_bprep");
}

int rot_tc_group(const RotJob *jobs_dev, int njobs, int64_t ntile, int64_t nrow, int *err, cudaStream_t st) {
  MK_CHECK_ARG(rot_tc_supported(nrow), "tensor-core rotation supports ndet in {32,64,128,256}, got %lld",
               (long long)nrow);
  MK_CHECK_ARG(jobs_dev && njobs >= 1 && err, "tensor-core rotation group: bad arguments");
  if (ntile <= 0) return MK_OK;
  const int nd = (int)nrow;
  const size_t wsmem = ws_smem_bytes(nd);
  int rc = ws_prepare(wsmem);
  if (rc) return rc;
  int64_t grid = (int64_t)sm_count();
  if (grid > ntile) grid = ntile;
  RotJob none{};
  k_rot_tc_ws<<<(unsigned)grid, WS_THREADS, wsmem, st>>>(jobs_dev, njobs, none, ntile, nd, err, 0, 1, 0);
  return launch_status("rot_tc_group");
}

}  // namespace mk
