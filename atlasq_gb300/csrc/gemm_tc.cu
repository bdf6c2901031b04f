// Batched complex GEMM on the 5th-generation tensor cores (sm_103a):
// D = alpha * op(A) op(B) + beta * Csrc, complex64, split precision 3xTF32.
//
// One CTA (9 warps) per 128 x 64 output tile, K in slices of 32:
//  * warps 0-7 (the converters) read the complex64 slice of op(A) (128 x 32)
//    and op(B)^T (64 x 32) straight from the operands with coalesced loads
//    (along k when k is contiguous in memory, along the rows otherwise), split
//    each value into TF32 hi = x rounded to TF32 (11-bit significand) and
//    lo = x - hi, fold conjugation into the imaginary parts, and store them
//    into a shared-memory stage in the K-major 128-byte-swizzled layout the
//    tensor core reads (the layout a TMA SWIZZLE_128B copy of 32-float rows
//    produces): A as four planes {Re_hi, Re_lo, Im_hi, Im_lo}, B as two
//    planes {hi, lo} of 192 rows [-Im | Re | Im]; out-of-range rows and k are
//    stored as zeros;
//  * warp 8 lane 0 issues tcgen05.mma.kind::tf32 (M=128, N=128, K=8) per stage,
//    the real and imaginary accumulators of the tile being adjacent TMEM
//    columns written by one MMA: with B rows 64..191 = [Re | Im] and rows
//    0..127 = [-Im | Re],
//       [Re | Im] += Ar_h [Br|Bi]_h + Ar_h [Br|Bi]_l + Ar_l [Br|Bi]_h
//                  + Ai_h [-Bi|Br]_h + Ai_h [-Bi|Br]_l + Ai_l [-Bi|Br]_h
//    (six MMAs per K=8 step, each accumulator receiving the same products in
//    the same order as twelve N=64 MMAs would), k slices rotating over four
//    accumulator pairs; a commit per stage frees the stage for the converters;
//  * warps 0-7 then read the accumulators with tcgen05.ld (warp w reads TMEM
//    lanes 32(w%4)..+31 = tile rows, columns 32(w/4)..+31) and write
//    alpha*C + beta*Csrc.
// The operands are read once per tile and never written back in split form:
// no packing pass and no packed copy in global memory.  The converters'
// shared-memory stores reach the tensor core through fence.proxy.async and the
// stage's full barrier.  Every mbarrier wait is bounded; on expiry the kernel
// records AGB_ERR_TIMEOUT in a device status word, waits (bounded) for the
// issued MMAs and frees its tensor memory.
#include "gemm.cuh"
#include "gemm_tc.cuh"

namespace {

constexpr int BM = 128, BN = 64, BK = 32, STAGES = 2;
constexpr int TILE_A = BM * BK * 4;                    // 16 KiB per plane
constexpr int B_ROWS = 3 * BN;                         // B plane rows: -Im | Re | Im
constexpr int TILE_B = B_ROWS * BK * 4;                // 24 KiB per plane (hi, lo)
constexpr int STAGE_BYTES = 4 * TILE_A + 2 * TILE_B;   // 112 KiB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr int NACC = 4;                                // k-tiles rotate over 4 accumulator pairs
constexpr int TMEM_COLS = 2 * BN * NACC;               // 512 columns: (Re, Im) x 4
constexpr int CONV_WARPS = 8;
constexpr int NCONV = 32 * CONV_WARPS;                 // converter / epilogue threads (warps 0-7)
constexpr int NTHREADS = NCONV + 32;                   // + warp 8: tensor memory and MMA issue
constexpr int MMA_WARP = CONV_WARPS;
constexpr int QA = BM * BK / 4 / NCONV, QB = BN * BK / 4 / NCONV;  // quads (4 consecutive k) per thread per k slice
constexpr unsigned WAIT_LIMIT = 1u << 26;              // bounded spin (~seconds)

AGB_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

AGB_DEV void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
AGB_DEV void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// true when phase `parity` of the barrier completed; false after `limit` polls
AGB_DEV bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned limit = WAIT_LIMIT) {
  const uint32_t a = smem_u32(bar);
  for (unsigned it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row atoms of
// 1024 B (stride byte offset), descriptor version 1.
AGB_DEV uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;             // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;   // stride byte offset
  d |= (uint64_t)1 << 46;             // version
  d |= (uint64_t)2 << 61;             // SWIZZLE_128B
  return d;
}
// Instruction descriptor, kind::tf32: D f32, A/B tf32, K-major, M=128, N=128
// (the real and imaginary accumulators of a tile are adjacent TMEM columns,
// written by one MMA).
constexpr uint32_t IDESC =
    (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)((2 * BN) >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);

AGB_DEV void umma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
AGB_DEV void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
AGB_DEV void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// x rounded to TF32 (10 explicit mantissa bits), round to nearest even.
AGB_DEV float tf32_hi(float x) {
  uint32_t b;
  asm("cvt.rn.tf32.f32 %0, %1;" : "=r"(b) : "f"(x));
  return __uint_as_float(b & 0xFFFFE000u);
}

// Byte offset of element (row r, k) in a plane tile of 128-byte rows (32 fp32)
// with the 128-byte swizzle: 16-byte chunk c of row r sits at chunk c ^ (r % 8)
// (the tile starts on a 1024-byte boundary).
AGB_DEV uint32_t sw128(int r, int k) { return (uint32_t)(r * 128 + (((k >> 2) ^ (r & 7)) << 4) + ((k & 3) << 2)); }

AGB_DEV void st_shared_v4(uint32_t addr, float a, float b, float c, float d) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

// A converter thread handles quads: 4 consecutive k of one row, which are
// one 16-byte chunk of the swizzled tile (one vector store per plane).  The
// j-th quad of thread ct:
//  * k contiguous in memory: a warp takes 4 rows x 32 k (lanes: row
//    lane / 8, quad lane % 8), rows 4 (w + 8 j) ..; each row is one 256-byte
//    read;
//  * otherwise: a warp takes 32 consecutive rows x one quad (lanes: row),
//    blocks b = w + 8 j with quad b % 8 and 32-row chunk b / 8; each k of the
//    quad is one 256-byte read.
// Either way each 8-lane phase of a vector store covers the 8 chunk positions
// of the 128-byte swizzle (chunk (k/4) ^ (row % 8)): no bank conflicts.
AGB_DEV void quad_coord(bool k_contig, int ct, int j, int& r, int& k4) {
  const int lane = ct & 31, w = ct >> 5;
  if (k_contig) {
    r = 4 * (w + CONV_WARPS * j) + (lane >> 3);
    k4 = 4 * (lane & 7);
  } else {
    const int b = w + CONV_WARPS * j;
    k4 = 4 * (b & 7);
    r = 32 * (b >> 3) + lane;
  }
}

// Element (row, k) of the operand as the MMA sees it:
//   A (which 0): op(A)[row][k];  B (which 1): op(B)[k][row]
// stored form: A op N/R -> A[row][k]; op T/C -> A[k][row]
//              B op N/R -> B[k][row]; op T/C -> B[row][k]
struct Operand {
  const float2* p;
  int64_t ld;
  int rows, K;
  bool k_contig, conj;
};
AGB_DEV Operand operand(const GemmProb& P, int which) {
  Operand o;
  const int op = which == 0 ? P.opA : P.opB;
  o.p = (const float2*)(which == 0 ? P.A : P.B);
  o.ld = which == 0 ? P.lda : P.ldb;
  o.rows = which == 0 ? P.M : P.N;
  o.K = P.K;
  const bool transposed = (op == 1 || op == 2);
  o.k_contig = (which == 0) ? !transposed : transposed;
  o.conj = (op == 2 || op == 3);
  return o;
}
template <int NQ>
AGB_DEV void load_slice(const Operand& o, int r0, int k0, int ct, float2* v) {
#pragma unroll
  for (int j = 0; j < NQ; ++j) {
    int r, k4;
    quad_coord(o.k_contig, ct, j, r, k4);
    r += r0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int k = k0 + k4 + t;
      float2 x = make_float2(0.f, 0.f);
      if (r < o.rows && k < o.K) x = o.k_contig ? o.p[(int64_t)r * o.ld + k] : o.p[(int64_t)k * o.ld + r];
      v[4 * j + t] = x;
    }
  }
}
// B quads: the hi and lo planes hold rows [-Im | Re | Im] (BN rows each), so
// rows BN..3BN-1 are the operand [Re | Im] of an A_re product and rows
// 0..2BN-1 the operand [-Im | Re] of an A_im product: one N = 2 BN MMA then
// accumulates both the real and the imaginary part of the tile.
template <int NQ>
AGB_DEV void store_slice_b(const Operand& o, uint32_t tile, int ct, const float2* v) {
#pragma unroll
  for (int j = 0; j < NQ; ++j) {
    int r, k4;
    quad_coord(o.k_contig, ct, j, r, k4);
    float rh[4], rl[4], ih[4], il[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const float re = v[4 * j + t].x, im = o.conj ? -v[4 * j + t].y : v[4 * j + t].y;
      rh[t] = tf32_hi(re);
      ih[t] = tf32_hi(im);
      rl[t] = re - rh[t];
      il[t] = im - ih[t];
    }
    const uint32_t a = tile + sw128(r, k4);  // rows r, r + BN, r + 2 BN share the swizzle phase
    constexpr uint32_t RB = BN * 128;
    st_shared_v4(a, -ih[0], -ih[1], -ih[2], -ih[3]);
    st_shared_v4(a + RB, rh[0], rh[1], rh[2], rh[3]);
    st_shared_v4(a + 2 * RB, ih[0], ih[1], ih[2], ih[3]);
    st_shared_v4(a + TILE_B, -il[0], -il[1], -il[2], -il[3]);
    st_shared_v4(a + TILE_B + RB, rl[0], rl[1], rl[2], rl[3]);
    st_shared_v4(a + TILE_B + 2 * RB, il[0], il[1], il[2], il[3]);
  }
}
template <int NQ>
AGB_DEV void store_slice(const Operand& o, uint32_t tile, int plane_bytes, int ct, const float2* v) {
#pragma unroll
  for (int j = 0; j < NQ; ++j) {
    int r, k4;
    quad_coord(o.k_contig, ct, j, r, k4);
    float rh[4], rl[4], ih[4], il[4];
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const float re = v[4 * j + t].x, im = o.conj ? -v[4 * j + t].y : v[4 * j + t].y;
      rh[t] = tf32_hi(re);
      ih[t] = tf32_hi(im);
      rl[t] = re - rh[t];
      il[t] = im - ih[t];
    }
    const uint32_t a = tile + sw128(r, k4);
    st_shared_v4(a, rh[0], rh[1], rh[2], rh[3]);
    st_shared_v4(a + plane_bytes, rl[0], rl[1], rl[2], rl[3]);
    st_shared_v4(a + 2 * plane_bytes, ih[0], ih[1], ih[2], ih[3]);
    st_shared_v4(a + 3 * plane_bytes, il[0], il[1], il[2], il[3]);
  }
}

// ------------------------------------------------------------------ GEMM
__global__ void __launch_bounds__(NTHREADS, 1)
    tc_gemm_kernel(const GemmProb* __restrict__ probs, int* __restrict__ status, unsigned pipe_limit) {
  const GemmProb P = probs[blockIdx.z];
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  if (m0 >= P.M || n0 >= P.N) return;
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* done = empty + STAGES;
  uint32_t* tmem_slot = (uint32_t*)(done + 1);
  volatile int* abort_flag = (volatile int*)(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nk = (P.K + BK - 1) / BK;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], NCONV);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  if (warp < CONV_WARPS) {
    // ---------------- converters: global complex64 -> split TF32 planes in shared memory
    const int ct = threadIdx.x;
    const Operand oa = operand(P, 0), ob = operand(P, 1);
    for (int kt = 0; kt < nk; ++kt) {
      const int s = kt % STAGES;
      float2 va[4 * QA], vb[4 * QB];
      load_slice<QA>(oa, m0, kt * BK, ct, va);  // in flight while the stage drains
      load_slice<QB>(ob, n0, kt * BK, ct, vb);
      if (kt >= STAGES && !mbar_wait(&empty[s], ((kt / STAGES) - 1) & 1, pipe_limit)) {
        *abort_flag = 1;
        break;
      }
      if (*abort_flag) break;
      const uint32_t st = smem_u32(smem + s * STAGE_BYTES);
      store_slice<QA>(oa, st, TILE_A, ct, va);
      store_slice_b<QB>(ob, st + 4 * TILE_A, ct, vb);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // visible to the tensor core
      mbar_arrive(&full[s]);
    }
  } else if (lane == 0) {
    // ---------------- MMA issuer
    // k-tile kt accumulates into pair kt % NACC: four chains of length K/4 instead
    // of one of length K (the tensor core's fp32 accumulation error grows with
    // the chain length); the epilogue sums the pairs in fp32.
    // Shared-memory descriptors: the address field is (address / 16) in the low
    // 14 bits, so a descriptor at a 16-byte multiple `off` past a stage base is
    // the base's descriptor + off / 16 (every operand lies below 256 KiB); the
    // two stage bases are formed once.
    static_assert(STAGES == 2, "two stage descriptors");
    const uint64_t dstage0 = sdesc(smem_u32(smem)), dstage1 = sdesc(smem_u32(smem + STAGE_BYTES));
    constexpr uint64_t A_PL = TILE_A >> 4, B0 = (4 * TILE_A) >> 4, B_LO = TILE_B >> 4, B_RE = (BN * 128) >> 4;
    for (int kt = 0; kt < nk; ++kt) {
      const int s = kt % STAGES;
      const uint32_t d = tmem + (uint32_t)(2 * BN * (kt % NACC));  // [re | im] columns of pair kt % NACC
      if (!mbar_wait(&full[s], (kt / STAGES) & 1, pipe_limit)) {
        *abort_flag = 1;
        break;
      }
      if (*abort_flag) break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint64_t ds = s ? dstage1 : dstage0;
#pragma unroll
      for (int ks = 0; ks < BK / 8; ++ks) {
        const uint64_t dk = ds + (uint64_t)(ks * 2);  // +32 bytes per K=8 step
        // A planes Re_hi, Re_lo, Im_hi, Im_lo; the [Re | Im] and [-Im | Re]
        // windows of the hi and lo B planes
        const uint64_t a0 = dk, a1 = dk + A_PL, a2 = dk + 2 * A_PL, a3 = dk + 3 * A_PL;
        const uint64_t bre_hi = dk + B0 + B_RE, bre_lo = dk + B0 + B_LO + B_RE;
        const uint64_t bim_hi = dk + B0, bim_lo = dk + B0 + B_LO;
        const uint32_t first = (kt < NACC && ks == 0) ? 0u : 1u;
        // re += Are Bre - Aim Bim,  im += Are Bim + Aim Bre  (3xTF32: hi hi, hi lo, lo hi)
        umma(d, a0, bre_hi, IDESC, first);
        umma(d, a0, bre_lo, IDESC, 1);
        umma(d, a1, bre_hi, IDESC, 1);
        umma(d, a2, bim_hi, IDESC, 1);
        umma(d, a2, bim_lo, IDESC, 1);
        umma(d, a3, bim_hi, IDESC, 1);
      }
      umma_commit(&empty[s]);  // stage s may be refilled once these MMAs retire
    }
    umma_commit(done);  // every MMA issued above has completed when this arrives
  }
  __syncwarp();
  // ---------------- epilogue (warps 0-7); the MMA warp waits for the MMAs before freeing TMEM.
  // This wait keeps the full limit even when the pipeline's is lowered, so an
  // aborted tile still retires every MMA it issued before TMEM is freed.
  const bool ok = mbar_wait(done, 0);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp < CONV_WARPS && ok && !*abort_flag) {
    const int quarter = warp & 3, half = warp >> 2;  // TMEM lanes 32 quarter.., columns 32 half..
    const int row = m0 + quarter * 32 + lane;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    float2* D = (float2*)P.D;
    const float2* C = (const float2*)P.Csrc;
    const float ar = (float)P.alpha_re, ai = (float)P.alpha_im, br = (float)P.beta_re, bi = (float)P.beta_im;
    const bool use_beta = (br != 0.f || bi != 0.f);
    const int nacc = nk < NACC ? nk : NACC;
#pragma unroll 1
    for (int c0 = half * (BN / 2); c0 < (half + 1) * (BN / 2); c0 += 16) {
      float re[16], im[16];
      tmem_ld16(tmem + lane_base + c0, re);
      tmem_ld16(tmem + lane_base + BN + c0, im);
      if (nk == 0) {
#pragma unroll
        for (int i = 0; i < 16; ++i) re[i] = im[i] = 0.f;  // empty inner dimension: product is zero
      }
      for (int a = 1; a < nacc; ++a) {
        float r2[16], i2[16];
        tmem_ld16(tmem + lane_base + (uint32_t)(2 * BN * a) + c0, r2);
        tmem_ld16(tmem + lane_base + (uint32_t)(2 * BN * a) + BN + c0, i2);
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          re[i] += r2[i];
          im[i] += i2[i];
        }
      }
      if (row < P.M) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int col = n0 + c0 + i;
          if (col < P.N) {
            float2 v = make_float2(ar * re[i] - ai * im[i], ar * im[i] + ai * re[i]);
            if (use_beta) {
              const float2 c = C[(int64_t)row * P.ldc + col];
              v.x += br * c.x - bi * c.y;
              v.y += br * c.y + bi * c.x;
            }
            D[(int64_t)row * P.ldd + col] = v;
          }
        }
      }
    }
  } else if (threadIdx.x == 0 && (!ok || *abort_flag)) {
    atomicExch(status, AGB_ERR_TIMEOUT);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
  }
}

int round_up(int x, int m) { return (x + m - 1) / m * m; }

unsigned g_pipe_limit = WAIT_LIMIT;

}  // namespace

// Poll limit of the GEMM's pipeline waits (stage full / empty); a negative value
// restores the default.  Lets a test make those waits expire: the kernel then
// reports AGB_ERR_TIMEOUT and skips its epilogue.
extern "C" int agb_set_gemm_wait_limit(long long polls) {
  g_pipe_limit = polls < 0 ? WAIT_LIMIT : (unsigned)(polls < (long long)WAIT_LIMIT ? polls : (long long)WAIT_LIMIT);
  return AGB_OK;
}

// The split operands live only in shared memory: the tensor-core path needs
// no global scratch beyond a token the dispatcher checks for.
size_t tc_gemm_scratch_bytes(int count, int maxM, int maxN, int maxK) {
  (void)count;
  (void)maxM;
  (void)maxN;
  (void)maxK;
  return 256;
}

int launch_gemm_tc(const GemmProb* probs, int count, int maxM, int maxN, int maxK, void* scratch,
                   size_t scratch_bytes, int* status, cudaStream_t s) {
  if (count <= 0 || maxM <= 0 || maxN <= 0) return AGB_OK;
  if (maxK <= 0) return AGB_ERR_ARG;
  if (count > 65535) return AGB_ERR_UNSUPPORTED;
  if (!scratch || scratch_bytes < tc_gemm_scratch_bytes(count, maxM, maxN, maxK)) return AGB_ERR_WORKSPACE;
  const int Mp = round_up(maxM, BM), Np = round_up(maxN, BN);
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(tc_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES) != cudaSuccess)
      return AGB_ERR_CUDA;
    attr = true;
  }
  tc_gemm_kernel<<<dim3(Np / BN, Mp / BM, count), NTHREADS, SMEM_BYTES, s>>>(probs, status, g_pipe_limit);
  AGB_CHECK_LAUNCH();
  return AGB_OK;
}

// Strided-batch host entry for the tensor-core GEMM (complex64).
namespace {
__global__ void strided_probs_kernel(GemmProb* out, GemmProb base, int count, int64_t sA, int64_t sB, int64_t sC) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  GemmProb p = base;
  p.A = (const float2*)base.A + (int64_t)i * sA;
  p.B = (const float2*)base.B + (int64_t)i * sB;
  p.D = (float2*)base.D + (int64_t)i * sC;
  p.Csrc = (const float2*)base.Csrc + (int64_t)i * sC;
  out[i] = p;
}
int opc(char c) {
  return (c == 'N' || c == 'n') ? 0 : (c == 'T' || c == 't') ? 1 : (c == 'C' || c == 'c') ? 2 : (c == 'R' || c == 'r') ? 3 : -1;
}
}  // namespace

extern "C" size_t agb_cgemm_tc_workspace(int batch, int M, int N, int K) {
  return agb_align((size_t)batch * sizeof(GemmProb)) + agb_align(sizeof(int)) + tc_gemm_scratch_bytes(batch, M, N, K);
}

// status_dev == NULL: the status word lives in the workspace, is cleared first,
// and (if status_host) is read back after a stream synchronisation.
// status_dev != NULL: the kernels record a timeout in *status_dev, which is
// never cleared here (sticky across calls), and nothing synchronises.
static int cgemm_tc_impl(char opA, char opB, int batch, int M, int N, int K, const void* A, int64_t lda,
                         int64_t strideA, const void* B, int64_t ldb, int64_t strideB, void* C, int64_t ldc,
                         int64_t strideC, float alpha_re, float alpha_im, float beta_re, float beta_im, void* ws,
                         size_t ws_bytes, int* status_host, int* status_dev, void* stream) {
  const int oa = opc(opA), ob = opc(opB);
  if (oa < 0 || ob < 0 || batch < 0 || M < 0 || N < 0 || K <= 0 || !ws) return AGB_ERR_ARG;
  if (batch == 0 || M == 0 || N == 0) return AGB_OK;
  if (ws_bytes < agb_cgemm_tc_workspace(batch, M, N, K)) return AGB_ERR_WORKSPACE;
  GemmProb base;
  base.A = A;
  base.B = B;
  base.D = C;
  base.Csrc = C;
  base.lda = lda;
  base.ldb = ldb;
  base.ldd = ldc;
  base.ldc = ldc;
  base.M = M;
  base.N = N;
  base.K = K;
  base.opA = oa;
  base.opB = ob;
  base.alpha_re = alpha_re;
  base.alpha_im = alpha_im;
  base.beta_re = beta_re;
  base.beta_im = beta_im;
  char* w = (char*)ws;
  GemmProb* probs = (GemmProb*)w;
  int* status = (int*)(w + agb_align((size_t)batch * sizeof(GemmProb)));
  void* scratch = w + agb_align((size_t)batch * sizeof(GemmProb)) + agb_align(sizeof(int));
  cudaStream_t s = (cudaStream_t)stream;
  if (status_dev) status = status_dev;
  else if (cudaMemsetAsync(status, 0, sizeof(int), s) != cudaSuccess) return AGB_ERR_CUDA;
  strided_probs_kernel<<<(batch + 127) / 128, 128, 0, s>>>(probs, base, batch, strideA, strideB, strideC);
  AGB_CHECK_LAUNCH();
  int rc = launch_gemm_tc(probs, batch, M, N, K, scratch, ws_bytes - (size_t)((char*)scratch - w), status, s);
  if (rc) return rc;
  if (status_host && !status_dev) {
    if (cudaMemcpyAsync(status_host, status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return AGB_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return AGB_ERR_CUDA;
    if (*status_host) return *status_host;
  }
  return AGB_OK;
}

extern "C" int agb_cgemm_tc(char opA, char opB, int batch, int M, int N, int K, const void* A, int64_t lda,
                            int64_t strideA, const void* B, int64_t ldb, int64_t strideB, void* C, int64_t ldc,
                            int64_t strideC, float alpha_re, float alpha_im, float beta_re, float beta_im, void* ws,
                            size_t ws_bytes, int* status_host, void* stream) {
  return cgemm_tc_impl(opA, opB, batch, M, N, K, A, lda, strideA, B, ldb, strideB, C, ldc, strideC, alpha_re,
                       alpha_im, beta_re, beta_im, ws, ws_bytes, status_host, nullptr, stream);
}

extern "C" int agb_cgemm_tc_async(char opA, char opB, int batch, int M, int N, int K, const void* A, int64_t lda,
                                  int64_t strideA, const void* B, int64_t ldb, int64_t strideB, void* C,
                                  int64_t ldc, int64_t strideC, float alpha_re, float alpha_im, float beta_re,
                                  float beta_im, void* ws, size_t ws_bytes, int* status_dev, void* stream) {
  if (!status_dev) return AGB_ERR_ARG;
  return cgemm_tc_impl(opA, opB, batch, M, N, K, A, lda, strideA, B, ldb, strideB, C, ldc, strideC, alpha_re,
                       alpha_im, beta_re, beta_im, ws, ws_bytes, nullptr, status_dev, stream);
}
