// Strided-line passes of the FP32 pair-solve pipeline on the packed two-line
// engine (fft2p.cuh): y forward, x forward * kernel * x inverse, y inverse.
//
// Work unit (tile): 2 LPR adjacent columns (LPR line pairs) of one outer index
// of one field. Thread (pr, q) transforms the two lines of pair pr, q being n2
// in stages 1/B and k1 in stages 2/A exactly as in fast::k_cols. The kernel is
// persistent: each CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...
// and stages every tile's input rows (and, in the x pass, its block of the
// kernel spectrum) in shared memory with TMA, one elected thread issuing the
// next tile's copies as soon as the current tile's input has been consumed,
// so the loads run under the current tile's transforms. Every wait is bounded.
//
// Layouts: the y-transformed spectral buffer (S2) is kept in the split pair
// layout (re_a, re_b, im_a, im_b) so the x pass reads register pairs
// directly; the y forward reads and the y inverse writes the complex rows
// (AoS) of S1 that the z passes use.
#pragma once
#include <atomic>

#include <cuda.h>

#include "fft2p.cuh"
#include "poisson_fast.cuh"
#include "ptx.cuh"

namespace gato {
namespace packed {

using fft2p::CP;

template <int R1, int R2, int LPR, int MODE>
struct PGeom {
  static constexpr int M = R1 * R2, N = M / 2, HH = M / 2 + 1;
  static constexpr int RM = R1 > R2 ? R1 : R2, NT = LPR * RM, CW = 2 * LPR;   // threads, columns per tile
  static constexpr int P = MODE == COL_INV ? M : N;            // staged input positions
  static constexpr int NSPLIT = (P + 255) / 256, PB = P / NSPLIT;   // TMA boxes <= 256 rows
  static_assert(P % NSPLIT == 0, "staged rows split into equal boxes");
  static constexpr uint32_t IN_BYTES = (uint32_t)P * CW * 8;
  static constexpr uint32_t G_BYTES = MODE == COL_FMI ? (uint32_t)HH * CW * 4 : 0;
  static constexpr int r128(int b) { return (b + 127) / 128 * 128; }
  // shared layout (bytes): stage | kernel spectrum x2 (x pass) | exchange buffer | twiddles
  static constexpr int OFF_G = r128(P * LPR * 16);
  static constexpr int G_SLOT = r128((int)G_BYTES);
  static constexpr int OFF_BUF = OFF_G + 2 * G_SLOT;
  static constexpr int OFF_TW = OFF_BUF + M * LPR * 16;
  // twiddle rows padded to R2 + 2 entries: the four k1 rows a warp reads start 8 banks apart,
  // so one 16-byte load of the warp (four distinct entries) is one shared-memory wavefront
  static constexpr int TWS = R2 + 2;
  static constexpr int SMEM = OFF_TW + R1 * TWS * 16 + 128;   // + slack to align the base to 128 bytes
};

// MODE: COL_FWD (S1 AoS in, S2 split out), COL_FMI (S2 in place), COL_INV (S2 in, S1 AoS out).
// tin: the input buffer as floats, dims {2 ncols, pos/outer axes, fields} (see LaunchP);
// tg (x pass): ghat2 as {M (kz), HH (kyo), HH (kxo)}.
template <int R1, int R2, int LPR, int MODE>
__global__ void __launch_bounds__(PGeom<R1, R2, LPR, MODE>::NT)
    k_colsp(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tg, float2* out,
            ColGeom g, int n_outer, int nf, const float4* tw4, int* err) {
  using G = PGeom<R1, R2, LPR, MODE>;
  constexpr int M = G::M, HH = G::HH, CW = G::CW, NT = G::NT;
  extern __shared__ __align__(128) unsigned char smdyn[];
  __shared__ __align__(8) uint64_t mbar[2];
  // TMA destinations on 128-byte boundaries: offset the base of the shared array itself
  unsigned char* smraw = smdyn + ((128u - (smem_u32(smdyn) & 127u)) & 127u);
  float4* stage = reinterpret_cast<float4*>(smraw);   // [pos][pair], as the tensor holds it
  float* gsp = reinterpret_cast<float*>(smraw + G::OFF_G);
  float4* buf = reinterpret_cast<float4*>(smraw + G::OFF_BUF);
  float4* tws = reinterpret_cast<float4*>(smraw + G::OFF_TW);
  const int t = threadIdx.x;
  const int pr = t % LPR, q = t / LPR;
  const int ncb = g.ncols / CW;
  const int ntiles = nf * n_outer * ncb;
  const int64_t ops = g.out_ps / 2;   // float4 units
  // tile -> (field fastest, then column block, then outer): the fields of one x-pass
  // (ky, column block) run side by side and share its kernel-spectrum block in L2
  auto decode = [&](int tile, int& f, int& cb, int& outer) {
    f = tile % nf;
    const int r = tile / nf;
    cb = r % ncb;
    outer = r / ncb;
  };
  auto issue = [&](int tile, int slot) {   // one thread: the tile's copies on mbar[slot]
    int f, cb, outer;
    decode(tile, f, cb, outer);
    mbar_expect_tx(&mbar[slot], G::IN_BYTES + G::G_BYTES);
    if (MODE == COL_FWD) {
      tma_load_4d(stage, &tin, &mbar[slot], cb * 2 * CW, 0, outer, f);
    } else if (MODE == COL_FMI) {
      tma_load_4d(stage, &tin, &mbar[slot], cb * 2 * CW, outer, 0, f);
      const int kyo = outer <= M - outer ? outer : M - outer;
      tma_load_3d(gsp + slot * (G::G_SLOT / 4), &tg, &mbar[slot], cb * CW, kyo, 0);
    } else {
#pragma unroll
      for (int s = 0; s < G::NSPLIT; ++s)
        tma_load_4d(stage + s * G::PB * LPR, &tin, &mbar[slot], cb * 2 * CW, s * G::PB, outer, f);
    }
  };
  if (t == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_barrier_init();
  }
  for (int i = t; i < R1 * R2; i += NT) tws[(i / R2) * G::TWS + i % R2] = tw4[i];
  __syncthreads();
  if (t == 0 && (int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int slot = it & 1;
    int f, cb, outer;
    decode(tile, f, cb, outer);
    const bool bad = !mbar_wait_bounded(&mbar[slot], (it >> 1) & 1, err, 111);
    if (__syncthreads_or(bad)) {
      // the copies of this tile may still be landing: the issuing thread waits for them
      // (bounded) before the CTA and its shared memory go away
      if (t == 0) mbar_wait_bounded(&mbar[slot], (it >> 1) & 1, err, 112);
      return;
    }
    float4* dst = reinterpret_cast<float4*>(out + f * g.out_fs + outer * g.out_os + cb * CW) + pr;
    CP X[R2];
    if (MODE != COL_INV) {
      if (q < R2) {
        CP v[R1];
#pragma unroll
        for (int n1 = 0; n1 < R1 / 2; ++n1) {
          const float4 w = stage[(R2 * n1 + q) * LPR + pr];
          v[n1] = MODE == COL_FWD ? fft2p::from_aos(w) : fft2p::from_split(w);
        }
        fft2p::rdft_half<R1, -1>(v);
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) buf[(q * R1 + k1) * LPR + pr] = fft2p::to_split(v[k1]);
      }
    } else if (q < R1) {
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) X[k2] = fft2p::from_split(stage[(q + R1 * k2) * LPR + pr]);
    }
    // the staged input (and the previous tile's kernel block) is consumed: the next tile's copies
    // may land on it once every thread's generic reads are ordered before the async proxy
    fence_proxy_async_smem();
    __syncthreads();
    if (t == 0 && tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x, slot ^ 1);
    if (MODE != COL_INV && q < R1) {
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) X[n2] = fft2p::from_split(buf[(n2 * R1 + q) * LPR + pr]);
      fft2p::twiddle_row<R2, -1>(X, tws + q * G::TWS);
      fft2p::rdft<R2, -1>(X);
      if (MODE == COL_FWD) {
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) dst[(int64_t)(q + R1 * k2) * ops] = fft2p::to_split(X[k2]);
      }
    }
    if (MODE == COL_FWD) {
      __syncthreads();   // stage-2 reads of buf are complete before the next tile's stage 1
      continue;
    }
    if (MODE == COL_FMI) {
      if (q < R1) {
        static_assert(R2 % 2 == 0, "the fold below splits k2 at R2 / 2");
        // kx = q + R1 k2: k2 < R2/2 reads row kx of the staged block, the upper half row M - kx
        const float* gs = gsp + slot * (G::G_SLOT / 4) + 2 * pr;
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) {
          const int kxo = k2 < R2 / 2 ? q + R1 * k2 : M - q - R1 * k2;
          const float2 gv = *reinterpret_cast<const float2*>(gs + kxo * CW);
          X[k2].re = fft2p::pmul(X[k2].re, gv);
          X[k2].im = fft2p::pmul(X[k2].im, gv);
        }
      }
      __syncthreads();   // stage-2 reads of buf are complete
    }
    if (q < R1) {
      fft2p::rdft<R2, +1>(X);
      fft2p::twiddle_row<R2, +1>(X, tws + q * G::TWS);
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) buf[(n2 * R1 + q) * LPR + pr] = fft2p::to_split(X[n2]);
    }
    __syncthreads();
    if (q < R2) {
      CP w[R1];
#pragma unroll
      for (int k1 = 0; k1 < R1; ++k1) w[k1] = fft2p::from_split(buf[(q * R1 + k1) * LPR + pr]);
      fft2p::rdft<R1, +1>(w);
#pragma unroll
      for (int n1 = 0; n1 < R1 / 2; ++n1)
        dst[(int64_t)(q + R2 * n1) * ops] = MODE == COL_INV ? fft2p::to_aos(w[n1]) : fft2p::to_split(w[n1]);
    }
    __syncthreads();   // stage-B reads of buf are complete before the next tile's stage 1
  }
}

template <int R1, int R2, int LPR>
struct LaunchP {
  static constexpr int M = R1 * R2, N = M / 2, HH = M / 2 + 1, CW = 2 * LPR;

  template <int MODE>
  static int launch(const CUtensorMap& tin, const CUtensorMap& tg, float2* out, const ColGeom& g, int outer,
                    int nf, const float4* tw4, cudaStream_t s) {
    using G = PGeom<R1, R2, LPR, MODE>;
    auto kern = k_colsp<R1, R2, LPR, MODE>;
    // one resident wave of persistent CTAs (blocks per SM from the occupancy calculator)
    // the resident blocks of one wave (blocks per SM x SMs), computed once; read by any thread
    static std::atomic<int> wave{0};
    GATO_TRY(fast::smem_attr(kern, G::SMEM));
    int w = wave.load();
    if (w == 0) {
      int dev = 0, sms = 0, per_sm = 0;
      GATO_CUDA_TRY(cudaGetDevice(&dev));
      GATO_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
      GATO_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, G::NT, G::SMEM));
      if (per_sm < 1) return fail(GATO_EUNSUPPORTED, "packed column pass: no resident CTA fits");
      w = per_sm * sms;
      wave.store(w);
    }
    const int64_t ntiles = (int64_t)nf * outer * (g.ncols / CW);
    const unsigned grid = (unsigned)std::min<int64_t>(ntiles, (int64_t)w);
    kern<<<grid, G::NT, G::SMEM, s>>>(tin, tg, out, g, outer, nf, tw4, device_error_word());
    GATO_LAUNCH_TRY();
    return GATO_OK;
  }

  // in: the pass's input buffer (S1 for the y forward, S2 otherwise), nfa fields allocated.
  static int cols(int mode, const float2* in, float2* out, const ColGeom& g, int outer, int nf,
                  const float4* tw4, const float* ghat2, cudaStream_t s) {
    if (g.ncols != M || g.ncols % CW != 0)
      return fail(GATO_EUNSUPPORTED, "packed column pass: columns must be the M = %d spectrum columns", M);
    alignas(64) unsigned char tm[128];
    alignas(64) unsigned char gm[128] = {};
    TmaBox b;
    b.rank = 4;
    b.dims[0] = 2 * (uint64_t)M;   // floats along the columns (kz)
    b.box[0] = 2 * CW;
    if (mode == COL_FWD) {         // S1[f][x][y < N][kz]: rows y of one x
      b.dims[1] = N;
      b.dims[2] = N;
      b.dims[3] = nf;
      b.strides_bytes[0] = (uint64_t)M * 8;
      b.strides_bytes[1] = (uint64_t)N * M * 8;
      b.strides_bytes[2] = (uint64_t)g.in_fs * 8;
      b.box[1] = N;
      b.box[2] = 1;
      b.box[3] = 1;
    } else {                       // S2[f][x < N][ky][kz]
      b.dims[1] = M;
      b.dims[2] = N;
      b.dims[3] = nf;
      b.strides_bytes[0] = (uint64_t)M * 8;
      b.strides_bytes[1] = (uint64_t)M * M * 8;
      b.strides_bytes[2] = (uint64_t)g.in_fs * 8;
      if (mode == COL_FMI) {       // rows x of one ky
        b.box[1] = 1;
        b.box[2] = N;
      } else {                     // rows ky of one x, in boxes of at most 256
        b.box[1] = PGeom<R1, R2, LPR, COL_INV>::PB;
        b.box[2] = 1;
      }
      b.box[3] = 1;
    }
    GATO_TRY(encode_tma(tm, GATO_F32, in, b));
    if (mode == COL_FMI) {
      TmaBox gb;
      gb.rank = 3;
      gb.dims[0] = M;
      gb.dims[1] = HH;
      gb.dims[2] = HH;
      gb.strides_bytes[0] = (uint64_t)M * 4;
      gb.strides_bytes[1] = (uint64_t)HH * M * 4;
      gb.box[0] = CW;
      gb.box[1] = 1;
      gb.box[2] = HH;
      GATO_TRY(encode_tma(gm, GATO_F32, ghat2, gb));
    }
    const CUtensorMap& T = *reinterpret_cast<const CUtensorMap*>(tm);
    const CUtensorMap& Gm = *reinterpret_cast<const CUtensorMap*>(gm);
    if (mode == COL_FWD) return launch<COL_FWD>(T, Gm, out, g, outer, nf, tw4, s);
    if (mode == COL_FMI) return launch<COL_FMI>(T, Gm, out, g, outer, nf, tw4, s);
    return launch<COL_INV>(T, Gm, out, g, outer, nf, tw4, s);
  }
};

}  // namespace packed
}  // namespace gato
