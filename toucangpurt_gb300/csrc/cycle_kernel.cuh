// GB300 (sm_103a) cycle kernel of the Toucan netlist evaluation: the device
// code shared by the translation units that instantiate its kernels
// (cycle_kernel.cu and kernels_{persistent,region}_{staged,resident}.cu).
//
// Restates the reference device code (src/SimEval.cu:304-1056) for many
// stimulus streams at once:
//   * one 32-bit word per value-pool slot carries the nibbles of 8 streams
//     (SPW = 8; SPW = 1 runs a single stream in nibble 0), so every
//     __shfl_sync of a micro-partition level moves 8 streams' operands and
//     the 4,642-entry truth table is indexed once per stream from shared
//     memory, where a cp.async.bulk copy staged it at kernel start (the
//     reference reads __constant__ memory with lane-divergent addresses,
//     SimEval.cu:190,354,411);
//   * a block evaluates G 8-stream groups of a partition together, giving G
//     independent dependency chains per warp level (G words per slot in
//     shared memory, read with one vector load);
//   * one persistent cooperative launch runs many cycles; regions are
//     separated by a software grid barrier whose waits are bounded by a
//     global-timer budget (timeouts set an error word instead of hanging);
//   * partitions are statically assigned to blocks and micro-partitions to
//     warps by the host schedule (greedy gate count or learned cost).
// All mutable device state (registers, exchange, memories) is read with
// L1-bypassing loads because other blocks write it between barriers.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>

#include "devimage.h"
#include "kernels.h"

namespace tgs {
namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t rep8(uint32_t v) { return v * 0x11111111u; }
__device__ __forceinline__ uint32_t nib(uint32_t w, uint32_t k) { return (w >> (4u * k)) & 0xFu; }

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long dmix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ void raiseErr(const KParams &p, uint32_t code, uint32_t a, uint32_t b, uint32_t c) {
  if (atomicCAS(p.err, 0u, code) == 0u) {
    p.errInfo[0] = code;
    p.errInfo[1] = a;
    p.errInfo[2] = b;
    p.errInfo[3] = c;
  }
}

// ---- shared memory -----------------------------------------------------------
// Every shared-memory access of the evaluation goes through these helpers with
// 32-bit shared-window addresses, so the compiler emits shared loads and
// stores.  (A pointer that may refer to shared or to global memory, such as
// an exec level that is staged or not, would otherwise compile to generic
// accesses with 64-bit address arithmetic.)  Stores carry a memory clobber;
// loads are volatile, so the compiler keeps them in order with the stores.
// Truth-table reads are the exception: the table is written once, before the
// block barrier that ends the block's set-up, and never again, so its loads
// are plain (not volatile) and the compiler may schedule them freely among
// the value-pool accesses (their addresses depend on operands read after
// the set-up, which keeps them after it).
__device__ __forceinline__ uint32_t ldsTab(uint32_t a) {
  uint32_t v;
  asm("ld.shared.u8 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ uint32_t ldsU32(uint32_t a) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}
__device__ __forceinline__ uint2 ldsV2(uint32_t a) {
  uint2 v;
  asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "r"(a));
  return v;
}
__device__ __forceinline__ uint4 ldsV4(uint32_t a) {
  uint4 v;
  asm volatile("ld.shared.v4.u32 {%0, %1, %2, %3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "r"(a));
  return v;
}
__device__ __forceinline__ void stsU32(uint32_t a, uint32_t v) {
  asm volatile("st.shared.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void stsV2(uint32_t a, uint2 v) {
  asm volatile("st.shared.v2.u32 [%0], {%1, %2};" ::"r"(a), "r"(v.x), "r"(v.y) : "memory");
}
__device__ __forceinline__ void stsV4(uint32_t a, uint4 v) {
  asm volatile("st.shared.v4.u32 [%0], {%1, %2, %3, %4};" ::"r"(a), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w) : "memory");
}

// Predicated (volatile) pair load: no access where c is false (0, 0 then).
__device__ __forceinline__ uint2 ldsV2If(uint32_t a, bool c) {
  uint2 v = make_uint2(0u, 0u);
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %3, 0;\n\t@q ld.shared.v2.u32 {%0, %1}, [%2];\n\t}"
               : "+r"(v.x), "+r"(v.y)
               : "r"(a), "r"(uint32_t(c)));
  return v;
}

// Words of a level block / micro-partition record: staged in shared memory
// (SH) or read from the schedule in global memory.
template <bool SH>
struct Words {
  const uint32_t *g;  // global address (SH = false)
  uint32_t s;         // shared address (SH = true)
  __device__ __forceinline__ uint32_t operator[](uint32_t i) const {
    if constexpr (SH) return ldsU32(s + 4u * i);
    else return __ldg(g + i);
  }
  // words i, i + 1 (i even: records are 16-byte aligned)
  __device__ __forceinline__ uint2 pair(uint32_t i) const {
    if constexpr (SH) return ldsV2(s + 4u * i);
    else return __ldg(reinterpret_cast<const uint2 *>(g + i));
  }
  // words i, i + 1 where c holds, (0, 0) elsewhere (no access)
  __device__ __forceinline__ uint2 pairIf(uint32_t i, bool c) const {
    if constexpr (SH) return ldsV2If(s + 4u * i, c);
    else return c ? __ldg(reinterpret_cast<const uint2 *>(g + i)) : make_uint2(0u, 0u);
  }
  __device__ __forceinline__ Words at(uint32_t off) const { return Words{g + off, s + 4u * off}; }
};

// value-pool slot word (slot, group) of a block's pool at shared address vp
template <int G>
__device__ __forceinline__ uint32_t vpAddr(uint32_t vp, uint32_t slot, uint32_t g) {
  return vp + 4u * (slot * uint32_t(G) + g);
}

// ---- truth-table lookup ---------------------------------------------------
// index = lutIndex + (a << 8 | b << 4 | c) per stream (SimEval.cu:353,410);
// tab = shared address of the staged table.
template <int SPW>
__device__ __forceinline__ uint32_t lookup(uint32_t tab, uint32_t base, uint32_t A, uint32_t B, uint32_t C);

template <>
__device__ __forceinline__ uint32_t lookup<1>(uint32_t tab, uint32_t base, uint32_t A, uint32_t B, uint32_t C) {
  return ldsTab(tab + base + (((A & 15u) << 8) | ((B & 15u) << 4) | (C & 15u)));
}

// prmt.b32 in its generic mode: a selector nibble with bit 3 set fills the
// result byte with the sign bit of the selected byte.  Applied to a byte
// below 0x80 it gives a zero byte, so one permute yields a zero-extended
// 12-bit index.
__device__ __forceinline__ uint32_t prmtIdx(uint32_t bc, uint32_t a, uint32_t sel) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(bc), "r"(a), "r"(sel));
  return d;
}

// 8 streams: even streams sit in the low nibble of each byte, odd streams in
// the high nibble.  (b << 4 | c) of 4 streams is formed per byte lane with
// masks; one permute per stream puts its a nibble above it (byte j of the bc
// and a words, upper half zero), and the 8 table bytes are packed back with
// permutes.
template <>
__device__ __forceinline__ uint32_t lookup<8>(uint32_t tab, uint32_t base, uint32_t A, uint32_t B, uint32_t C) {
  const uint32_t t = tab + base;
  const uint32_t bcE = ((B & 0x0F0F0F0Fu) << 4) | (C & 0x0F0F0F0Fu);
  const uint32_t bcO = (B & 0xF0F0F0F0u) | ((C >> 4) & 0x0F0F0F0Fu);
  const uint32_t aE = A & 0x0F0F0F0Fu, aO = (A >> 4) & 0x0F0F0F0Fu;
  // selector for byte j: result bytes (bc.j, a.j, sign(a.j), sign(a.j))
  const uint32_t r0 = ldsTab(t + prmtIdx(bcE, aE, 0xCC40u)), r2 = ldsTab(t + prmtIdx(bcE, aE, 0xDD51u));
  const uint32_t r4 = ldsTab(t + prmtIdx(bcE, aE, 0xEE62u)), r6 = ldsTab(t + prmtIdx(bcE, aE, 0xFF73u));
  const uint32_t r1 = ldsTab(t + prmtIdx(bcO, aO, 0xCC40u)), r3 = ldsTab(t + prmtIdx(bcO, aO, 0xDD51u));
  const uint32_t r5 = ldsTab(t + prmtIdx(bcO, aO, 0xEE62u)), r7 = ldsTab(t + prmtIdx(bcO, aO, 0xFF73u));
  const uint32_t lo = __byte_perm(__byte_perm(r0, r2, 0x0040), __byte_perm(r4, r6, 0x0040), 0x5410);
  const uint32_t hi = __byte_perm(__byte_perm(r1, r3, 0x0040), __byte_perm(r5, r7, 0x0040), 0x5410);
  return lo | (hi << 4);
}

// ---- value-pool words of G groups ----------------------------------------
template <int G>
__device__ __forceinline__ void loadG(uint32_t sa, uint32_t (&v)[G]) {
  if constexpr (G == 8) {
    const uint4 q = ldsV4(sa), r = ldsV4(sa + 16u);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    v[4] = r.x; v[5] = r.y; v[6] = r.z; v[7] = r.w;
  } else if constexpr (G == 4) {
    const uint4 q = ldsV4(sa);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
  } else if constexpr (G == 2) {
    const uint2 q = ldsV2(sa);
    v[0] = q.x; v[1] = q.y;
  } else {
    v[0] = ldsU32(sa);
  }
}

template <int G>
__device__ __forceinline__ void storeG(uint32_t sa, const uint32_t (&v)[G]) {
  if constexpr (G == 8) {
    stsV4(sa, make_uint4(v[0], v[1], v[2], v[3]));
    stsV4(sa + 16u, make_uint4(v[4], v[5], v[6], v[7]));
  } else if constexpr (G == 4) {
    stsV4(sa, make_uint4(v[0], v[1], v[2], v[3]));
  } else if constexpr (G == 2) {
    stsV2(sa, make_uint2(v[0], v[1]));
  } else {
    stsU32(sa, v[0]);
  }
}

// global (mutable state, L1 bypass) -> value pool
template <int G>
__device__ __forceinline__ void copyInG(uint32_t dst, const uint32_t *__restrict__ src) {
  if constexpr (G == 8) {
    stsV4(dst, __ldcg(reinterpret_cast<const uint4 *>(src)));
    stsV4(dst + 16u, __ldcg(reinterpret_cast<const uint4 *>(src) + 1));
  } else if constexpr (G == 4) {
    stsV4(dst, __ldcg(reinterpret_cast<const uint4 *>(src)));
  } else if constexpr (G == 2) {
    stsV2(dst, __ldcg(reinterpret_cast<const uint2 *>(src)));
  } else {
    stsU32(dst, __ldcg(src));
  }
}

// value pool -> global
template <int G>
__device__ __forceinline__ void copyOutG(uint32_t *__restrict__ dst, uint32_t src) {
  if constexpr (G == 8) {
    reinterpret_cast<uint4 *>(dst)[0] = ldsV4(src);
    reinterpret_cast<uint4 *>(dst)[1] = ldsV4(src + 16u);
  } else if constexpr (G == 4) {
    *reinterpret_cast<uint4 *>(dst) = ldsV4(src);
  } else if constexpr (G == 2) {
    *reinterpret_cast<uint2 *>(dst) = ldsV2(src);
  } else {
    *dst = ldsU32(src);
  }
}

// ---- word-wide top-level ops (records with kMPFastTop) ----------------------
// The op's table row is a bitwise function g of (b, c) -- checked against the
// table at load time -- so the 8 streams of a word take
//   out = Q ^ (C & (P ^ Q)),  P = g01 ^ (B & (g11 ^ g01)),  Q = g00 ^ (B & (g10 ^ g00))
// (g_xy: all ones where g(x, y) = 1), three bitwise instructions.  A
// multiplexer (kind 1: a ? b : c, kind 2: a ? c : b) starts from the pass-c
// (pass-b) row and blends in the other operand where the select nibble is 1;
// a word with a select nibble above 1 reads the table window instead.
template <int H>
__device__ __forceinline__ void fastTop(uint32_t tab, uint32_t lut, uint32_t kind, uint32_t g, const uint32_t (&A)[H],
                                        const uint32_t (&B)[H], const uint32_t (&C)[H], uint32_t (&v)[H], bool anySel) {
  g = kind == 0u ? g : kind == 1u ? kGPassC : kGPassB;
  const uint32_t g00 = 0u - (g & 1u), g01 = 0u - ((g >> 1) & 1u), g10 = 0u - ((g >> 2) & 1u), g11 = 0u - (g >> 3);
  const uint32_t k1 = g11 ^ g01, k0 = g10 ^ g00;
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const uint32_t P = (B[i] & k1) ^ g01, Q = (B[i] & k0) ^ g00;
    v[i] = Q ^ (C[i] & (P ^ Q));
  }
  if (anySel && kind != 0u) {
#pragma unroll
    for (int i = 0; i < H; ++i) {
      if ((A[i] & 0xEEEEEEEEu) == 0u) {  // every select nibble of the word is 0 or 1
        const uint32_t m = (A[i] & 0x11111111u) * 15u;
        const uint32_t X = kind == 1u ? B[i] : C[i];
        v[i] ^= m & (X ^ v[i]);
      } else {
        v[i] = lookup<8>(tab, lut, A[i], B[i], C[i]);
      }
    }
  }
}

// ---- micro-partitions (evalSingleMicroPart, SimEval.cu:304-580) -----------
// One pass of a LUT micro-partition over H stream groups starting at group
// h0 of the item (value-pool words [slot][G]).
template <int SPW, int G, int H, bool SH>
__device__ __forceinline__ void evalLutPass(const Words<SH> mp, uint32_t hdr, uint32_t vp, uint32_t tab, uint32_t lane,
                                            bool constSlots, uint32_t h0) {
  const uint32_t W = (hdr >> 2) & 63u, nMid = (hdr >> 8) & 255u, nWB = (hdr >> 16) & 63u;
  const Words<SH> top = mp.at(kMPHeaderWords);
  uint32_t v[H];
  uint32_t cres = 0;  // compact records: the lane's write-back slot
  // top level: operands < 16 are immediates, else value-pool slots
  if (lane < W) {
    const uint2 t = top.pair(2u * lane);
    // compact lanes (uniform per record) carry the write-back slot
    const bool compact = (hdr & kMPCompact) != 0u;
    uint32_t lut = compact ? t.y >> 16 : t.x & 0xFFFFu, a = compact ? t.x & 0xFFFu : t.x >> 16;
    const uint32_t b = compact ? (t.x >> 12) & 0xFFFu : t.y & 0xFFFFu;
    const uint32_t c = compact ? (t.x >> 24) | ((t.y & 15u) << 8) : t.y >> 16;
    cres = (t.y >> 4) & 0xFFFu;
    // word-wide record (uniform per record): the fast form for 8 streams
    // per word, the table form (lutIndex, op0) otherwise
    const bool fastRec = (hdr & kMPFastTop) != 0u;
    uint32_t kind = 0, fg = 0;
    if (fastRec) {
      kind = (lut >> kFastKindShift) & 3u;
      lut &= 0x1FFFu;
      if (kind == 0u) {
        fg = (a >> 4) & 15u;
        a &= 15u;
      }
    }
    uint32_t A[H], B[H], C[H];
    // a word-wide record without multiplexers never reads op0
    const bool needA = !(SPW == 8 && fastRec && !(hdr & kMPFastSel));
    if (constSlots) {
      if (needA) loadG<H>(vpAddr<G>(vp, a, h0), A);
      else {
#pragma unroll
        for (int g = 0; g < H; ++g) A[g] = 0u;
      }
      loadG<H>(vpAddr<G>(vp, b, h0), B);
      loadG<H>(vpAddr<G>(vp, c, h0), C);
    } else {
      if (a < 16) {
#pragma unroll
        for (int g = 0; g < H; ++g) A[g] = rep8(a);
      } else {
        loadG<H>(vpAddr<G>(vp, a, h0), A);
      }
      if (b < 16) {
#pragma unroll
        for (int g = 0; g < H; ++g) B[g] = rep8(b);
      } else {
        loadG<H>(vpAddr<G>(vp, b, h0), B);
      }
      if (c < 16) {
#pragma unroll
        for (int g = 0; g < H; ++g) C[g] = rep8(c);
      } else {
        loadG<H>(vpAddr<G>(vp, c, h0), C);
      }
    }
    if (SPW == 8 && fastRec) {
      fastTop<H>(tab, lut, kind, fg, A, B, C, v, (hdr & kMPFastSel) != 0);
    } else {
#pragma unroll
      for (int g = 0; g < H; ++g) v[g] = lut ? lookup<SPW>(tab, lut, A[g], B[g], C[g]) : C[g];
    }
  } else {
#pragma unroll
    for (int g = 0; g < H; ++g) v[g] = 0;
  }
  // middle levels: operand < 32 immediate, 32..63 = lane (op - 32) of the previous level
  const Words<SH> mid = top.at(2u * W);
  // each level's op word is read one level ahead, so its latency overlaps
  // the previous level's shuffles and lookups
  uint32_t wNext = nMid && lane < W ? mid[lane] : 0u;
  for (uint32_t m = 0; m < nMid; ++m) {
    const uint32_t w = wNext;
    wNext = m + 1 < nMid && lane < W ? mid[(m + 1) * W + lane] : 0u;
    const uint32_t c6 = w & 63u, b6 = (w >> 6) & 63u, a6 = (w >> 12) & 63u, lut = w >> 18;
    uint32_t nv[H];
#pragma unroll
    for (int g = 0; g < H; ++g) {
      const uint32_t As = __shfl_sync(kFull, v[g], int(a6 & 31u));
      const uint32_t Bs = __shfl_sync(kFull, v[g], int(b6 & 31u));
      const uint32_t Cs = __shfl_sync(kFull, v[g], int(c6 & 31u));
      const uint32_t A = a6 < 32 ? rep8(a6) : As;
      const uint32_t B = b6 < 32 ? rep8(b6) : Bs;
      const uint32_t C = c6 < 32 ? rep8(c6) : Cs;
      nv[g] = lut ? lookup<SPW>(tab, lut, A, B, C) : C;
    }
#pragma unroll
    for (int g = 0; g < H; ++g) v[g] = nv[g];
  }
  // write-back (SimEval.cu:422-447): shuffleId < 32 immediate, else lane
  // (shuffleId mod 32); a compact record's lane l writes its own value
  if (hdr & kMPCompact) {
    if (lane < nWB) storeG<H>(vpAddr<G>(vp, cres, h0), v);
    return;
  }
  const Words<SH> wb = mid.at(nMid * W);
  const uint32_t wv = lane < nWB ? wb[lane] : 0u;
  const uint32_t src = wv & 0xFFu, res = wv >> 16;
  if (hdr & kMPDirectWB) {  // entry l takes lane l's value: no exchange (uniform per record)
    if (lane < nWB) storeG<H>(vpAddr<G>(vp, res, h0), v);
    return;
  }
  uint32_t out[H];
#pragma unroll
  for (int g = 0; g < H; ++g) {
    const uint32_t x = __shfl_sync(kFull, v[g], int(src & 31u));
    out[g] = src < 32 ? rep8(src) : x;
  }
  if (lane < nWB) storeG<H>(vpAddr<G>(vp, res, h0), out);
}

// constSlots: value-pool slots 0..15 hold the immediates 0..15 (renumbered
// pools never use them), so operands are loaded without a branch.  More than
// 4 groups run as passes of 4 (the record is read once per pass from shared
// memory; the unit's bookkeeping is paid once).
template <int SPW, int G, bool SH>
__device__ __forceinline__ void evalLut(const Words<SH> mp, uint32_t hdr, uint32_t vp, uint32_t tab, uint32_t lane,
                                        bool constSlots) {
  constexpr int H = G > 4 ? 4 : G;
#pragma unroll 1
  for (uint32_t h0 = 0; h0 < uint32_t(G); h0 += H) evalLutPass<SPW, G, H, SH>(mp, hdr, vp, tab, lane, constSlots, h0);
}

// Special micro-partitions run on the stream groups [g0, g0 + gn) of the
// item: the schedule may give the groups of one micro-partition to several
// warps (a level of one special micro-partition would leave the other warps
// idle).
template <int SPW, int G, bool SH>
__device__ __forceinline__ void evalVecRead(const KParams &p, const PartDesc &d, const Words<SH> mp, uint32_t hdr,
                                            uint32_t vp, uint32_t lane, uint32_t g0, uint32_t gn) {
  const uint32_t n = (hdr >> 2) & 63u;
  if (lane >= n) return;
  const Words<SH> r = mp.at(kMPHeaderWords + lane * kVecReadWords);
  const uint32_t w0 = r[0], w1 = r[1], w2 = r[2], w3 = r[3], w4 = r[4];
  const uint32_t base = w0 & 0xFFFFu, len = w0 >> 16, off = w1 & 0xFFFFu, isConst = (w1 >> 16) & 1u;
  const uint32_t ix[4] = {w2 & 0xFFFFu, w2 >> 16, w3 & 0xFFFFu, w3 >> 16};
  const uint32_t outR = w4 & 0xFFFFu, res = w4 >> 16;
  const uint8_t *cv = p.constVec + d.constOff;
#pragma unroll 1
  for (uint32_t g = g0; g < g0 + gn; ++g) {
    uint32_t I[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) I[j] = ix[j] < 16 ? rep8(ix[j]) : ldsU32(vpAddr<G>(vp, ix[j], g));
    const uint32_t OR = outR < 16 ? rep8(outR) : ldsU32(vpAddr<G>(vp, outR, g));
    // the SPW reads of a word are issued before any is used
    uint32_t raw[SPW];
#pragma unroll
    for (int k = 0; k < SPW; ++k) {
      const uint32_t o = ((nib(I[0], k) << 12) | (nib(I[1], k) << 8) | (nib(I[2], k) << 4) | nib(I[3], k)) + off;
      if (o < len) raw[k] = isConst ? uint32_t(__ldg(cv + base + o)) : nib(ldsU32(vpAddr<G>(vp, base + o, g)), k);
      else raw[k] = nib(OR, k);
    }
    uint32_t out = 0;
#pragma unroll
    for (int k = 0; k < SPW; ++k) out |= (raw[k] & 15u) << (4 * k);
    stsU32(vpAddr<G>(vp, res, g), out);
  }
}

// Signed vector arithmetic on up to 31 nibbles per stream (SimEval.cu:482-548):
// nibble i of the vector sits in slot base + i, sign bit at 4 * len - 1.
// Work item = (op, group, stream), one per lane: the SPW lanes of one (op,
// group) hold the streams of one word and merge their result nibbles with
// shuffles, so no lane runs the streams of a word one after another.
// Vectors of up to 16 nibbles (the usual 32- and 64-bit ones) compute in
// 64-bit registers: after sign extension to 64 bits every value lies in
// [-2^63, 2^63), so the comparisons equal the reference's 128-bit ones, and
// sums, differences and products agree with them in the low 64 bits, which
// hold every result nibble (i < len <= 16).  Longer vectors take 128-bit
// arithmetic as the reference does.
template <int SPW, int G, bool SH>
__device__ void evalVecOp(const KParams &p, const PartDesc &d, const Words<SH> mp, uint32_t hdr, uint32_t vp,
                          uint32_t lane, uint32_t g0, uint32_t gn) {
  const uint32_t n = (hdr >> 2) & 63u;
  const uint32_t total = n * gn * SPW;
  const uint8_t *cv = p.constVec + d.constOff;
#pragma unroll 1
  for (uint32_t base = 0; base < total; base += 32) {  // the same trip count in every lane
    const uint32_t w = base + lane;
    const bool act = w < total;
    const uint32_t op = act ? w / (gn * SPW) : 0u;
    const uint32_t g = g0 + (w / SPW) % gn, k = w % SPW;
    const Words<SH> r = mp.at(kMPHeaderWords + op * kVecOpWords);
    const uint32_t w0 = r[0], w1 = r[1], res = r[2];
    const uint32_t v1 = w0 & 0xFFFFu, v2 = w0 >> 16, len = act ? (w1 & 0xFFFFu) : 0u, opc = (w1 >> 16) & 0xFFu;
    const uint32_t cf = w1 >> 24;
    const bool c1 = (cf & 2u) != 0, c2 = (cf & 1u) != 0;
    const bool isVec = opc <= 2;
    const bool narrow = len <= 16u;
    auto nibA = [&](uint32_t i) {
      return c1 ? (uint32_t(__ldg(cv + v1 + i)) & 15u) : nib(ldsU32(vpAddr<G>(vp, v1 + i, g)), k);
    };
    auto nibB = [&](uint32_t i) {
      return c2 ? (uint32_t(__ldg(cv + v2 + i)) & 15u) : nib(ldsU32(vpAddr<G>(vp, v2 + i, g)), k);
    };
    unsigned long long r64 = 0;
    unsigned __int128 rv = 0;
    if (narrow) {
      unsigned long long a = 0, b = 0;
#pragma unroll 4
      for (uint32_t i = 0; i < len; ++i) {
        a |= (unsigned long long)nibA(i) << (4 * i);
        b |= (unsigned long long)nibB(i) << (4 * i);
      }
      if (len) {
        const uint32_t s = 64u - 4u * len;  // sign extension from bit 4 * len - 1
        const long long sa = (long long)(a << s) >> s, sb = (long long)(b << s) >> s;
        switch (opc) {
          case 0: r64 = (unsigned long long)sa + (unsigned long long)sb; break;
          case 1: r64 = (unsigned long long)sa - (unsigned long long)sb; break;
          case 2: r64 = (unsigned long long)sa * (unsigned long long)sb; break;
          case 3: r64 = sa == sb; break;
          case 4: r64 = sa < sb; break;
          case 5: r64 = sa <= sb; break;
          default: r64 = 0; break;
        }
      }
    } else {
      unsigned __int128 a = 0, b = 0;
      for (uint32_t i = 0; i < len; ++i) {
        a |= (unsigned __int128)nibA(i) << (4 * i);
        b |= (unsigned __int128)nibB(i) << (4 * i);
      }
      const uint32_t sign = 4 * len - 1;
      if ((a >> sign) & 1) a |= ~(((unsigned __int128)1 << (sign + 1)) - 1);
      if ((b >> sign) & 1) b |= ~(((unsigned __int128)1 << (sign + 1)) - 1);
      const __int128 sa = (__int128)a, sb = (__int128)b;
      switch (opc) {
        case 0: rv = a + b; break;
        case 1: rv = a - b; break;
        case 2: rv = a * b; break;
        case 3: rv = sa == sb; break;
        case 4: rv = sa < sb; break;
        case 5: rv = sa <= sb; break;
        default: rv = 0; break;
      }
    }
    // result nibbles: len slots for arithmetic, one slot for a comparison
    const uint32_t outLen = act ? (isVec ? len : 1u) : 0u;
    uint32_t maxLen = outLen;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) maxLen = max(maxLen, __shfl_xor_sync(kFull, maxLen, o));
    for (uint32_t i = 0; i < maxLen; ++i) {
      const uint32_t x = narrow ? uint32_t(r64 >> (4 * (i & 15u))) : uint32_t(rv >> (4 * i));
      uint32_t word = i < outLen ? (x & 15u) << (4 * k) : 0u;
#pragma unroll
      for (int o = 1; o < SPW; o <<= 1) word |= __shfl_xor_sync(kFull, word, o);
      if (k == 0 && i < outLen) stsU32(vpAddr<G>(vp, (res + i) & 0xFFFFu, g), word);
    }
  }
}

// Memory reads (SimEval.cu:550-575): the loads of the SPW streams of a word
// are issued together, then merged.
template <int SPW, int G, bool SH>
__device__ __forceinline__ void evalMemRead(const KParams &p, const Words<SH> mp, uint32_t hdr, uint32_t vp,
                                            uint32_t lane, uint32_t gb, uint32_t g0, uint32_t gn) {
  const uint32_t n = (hdr >> 2) & 63u;
  if (lane >= n) return;
  const Words<SH> r = mp.at(kMPHeaderWords + lane * kMemReadWords);
  const uint32_t lo = r[0], hi = r[1], w2 = r[2], res = r[3];
  const unsigned long long memBase = (unsigned long long)lo | ((unsigned long long)(hi & 0x7FFFFFFFu) << 32);
  const bool multi = (hi >> 31) != 0;
  const uint32_t en = w2 & 0xFFFFu, av = w2 >> 16;
  if (en == 0) return;  // immediate 0: neither reads nor writes (SimEval.cu:559-560)
#pragma unroll 1
  for (uint32_t g = g0; g < g0 + gn; ++g) {
    const uint32_t EN = en < 16 ? rep8(en) : ldsU32(vpAddr<G>(vp, en, g));
    uint32_t AD[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) AD[j] = ldsU32(vpAddr<G>(vp, av + j, g));
    uint32_t out = ldsU32(vpAddr<G>(vp, res, g));  // a disabled read leaves the slot as it is
    // every stream's load is issued (predicated) before any is used, and an
    // out-of-range address is reported after them, so the SPW loads of a
    // word overlap instead of waiting one after another
    uint32_t val[SPW];
    uint32_t badK = SPW;
    unsigned long long badIdx = 0;
#pragma unroll
    for (int k = 0; k < SPW; ++k) {
      const uint32_t s = (gb * G + g) * SPW + k;
      uint32_t addr = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) addr |= nib(AD[j], k) << (4 * j);
      if (multi) addr <<= 2;
      const unsigned long long idx = memBase + addr;
      const bool on = s < p.nStreams && nib(EN, k) != 0, ok = on && idx < p.memPoolSize;
      if (on && !ok && badK == SPW) {
        badK = uint32_t(k);
        badIdx = idx;
      }
      val[k] = ok ? uint32_t(__ldcg(p.mems + s * p.memStride + idx)) : 0xFFu;  // 0xFF: no load
    }
    if (badK != SPW) raiseErr(p, kErrMemRange, uint32_t(badIdx), uint32_t(badIdx >> 32), (gb * G + g) * SPW + badK);
#pragma unroll
    for (int k = 0; k < SPW; ++k)
      if (val[k] != 0xFFu) out = (out & ~(15u << (4 * k))) | ((val[k] & 15u) << (4 * k));
    stsU32(vpAddr<G>(vp, res, g), out);
  }
}

// ---- exec-level staging ------------------------------------------------------
// Two shared-memory buffers: level lv + 1 is copied into one while level lv
// runs from the other (stageCopy below).  mb0 is the block's setup mbarrier
// (resident exec levels).
struct Stage {
  uint32_t buf0;   // shared address of buffer 0; buffer b at buf0 + b * bytes
  uint32_t bytes;  // bytes of one buffer
  uint32_t mb0;    // shared address of mbarrier 0
};

// A waiting thread is suspended by the hardware (up to this many ns per try)
// instead of spinning: no issue slots are spent on the wait.
constexpr uint32_t kStageSuspendNs = 20000;

// Staging: the threads of one warp copy the 16-byte pieces of a level block
// global -> shared with asynchronous copies through the load / store path
// (no copy engine, no mbarrier); a thread waits for its own copies right
// before the block barrier that opens the level, which then makes every
// piece visible to every thread.  (Level blocks are whole 16-byte units at
// 16-byte aligned offsets.)
__device__ __forceinline__ void stageCopy(const Stage &st, uint32_t b, const uint32_t *src, uint32_t words,
                                          uint32_t tid, uint32_t nthr) {
  const uint32_t dst = st.buf0 + b * st.bytes;
  for (uint32_t k = tid; k < words / 4u; k += nthr)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 16u * k), "l"(src + 4u * k) : "memory");
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void stageCopyWait() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// The units a warp runs in one exec level (block = the level's words).
// Unit u of a level block (unit word: record offset | first group << 24 |
// (groups - 1) << 27).
template <int SPW, int G, bool SH>
__device__ __forceinline__ void runUnit(const KParams &p, const PartDesc &d, const Words<SH> blk, const Words<SH> units,
                                        uint32_t u, uint32_t vp, uint32_t tab, uint32_t lane, uint32_t gb) {
  const uint32_t uw = units[u];
  const Words<SH> mp = blk.at(uw & kUnitOffsetMask);
  const uint32_t hdr = mp[0];
  if ((hdr & 3u) == kMPLut) {
    evalLut<SPW, G, SH>(mp, hdr, vp, tab, lane, p.constSlots != 0);  // always every group
  } else {
    const uint32_t g0 = (uw >> 24) & 7u, gn = ((uw >> 27) & 7u) + 1u;
    if ((hdr & 3u) == kMPVecRead) evalVecRead<SPW, G, SH>(p, d, mp, hdr, vp, lane, g0, gn);
    else if ((hdr & 3u) == kMPVecOp) evalVecOp<SPW, G, SH>(p, d, mp, hdr, vp, lane, g0, gn);
    else evalMemRead<SPW, G, SH>(p, mp, hdr, vp, lane, gb, g0, gn);
  }
  __syncwarp();
}

// A warp's units [ub, ue) of one level of a one-group item, each unit's
// record decoded while the previous one runs (defined with the one-group
// helpers below).
template <int SPW, bool SH>
__device__ __forceinline__ void runUnitsOne(const KParams &p, const PartDesc &d, const Words<SH> blk,
                                            const Words<SH> units, uint32_t ub, uint32_t ue, uint32_t vp, uint32_t tab,
                                            uint32_t lane, uint32_t gb);

template <int SPW, int G, bool SH>
__device__ __forceinline__ void runLevel(const KParams &p, const PartDesc &d, const Words<SH> blk, uint32_t vp,
                                         uint32_t tab, uint32_t lane, uint32_t warp, uint32_t NW, uint32_t gb) {
  const uint32_t ub = blk[1 + warp], ue = blk[2 + warp];
  const Words<SH> units = blk.at(2 + NW);
  if (!(p.flags & kFlagProfileMP)) {
    if constexpr (G == 1)
      runUnitsOne<SPW, SH>(p, d, blk, units, ub, ue, vp, tab, lane, gb);
    else
      for (uint32_t u = ub; u < ue; ++u) runUnit<SPW, G, SH>(p, d, blk, units, u, vp, tab, lane, gb);
    return;
  }
  // the same with clock64 around every unit (cost-model samples)
  for (uint32_t u = ub; u < ue; ++u) {
    const uint32_t uw = units[u];
    const Words<SH> mp = blk.at(uw & kUnitOffsetMask);
    const uint32_t g0 = (uw >> 24) & 7u, gn = ((uw >> 27) & 7u) + 1u;
    const uint32_t hdr = mp[0];
    const long long tm = clock64();
    switch (hdr & 3u) {
      case kMPLut: evalLut<SPW, G, SH>(mp, hdr, vp, tab, lane, p.constSlots != 0); break;
      case kMPVecRead: evalVecRead<SPW, G, SH>(p, d, mp, hdr, vp, lane, g0, gn); break;
      case kMPVecOp: evalVecOp<SPW, G, SH>(p, d, mp, hdr, vp, lane, g0, gn); break;
      default: evalMemRead<SPW, G, SH>(p, mp, hdr, vp, lane, gb, g0, gn); break;
    }
    __syncwarp();
    if (lane == 0) {
      const uint32_t id = mp[1];
      atomicAdd(p.mpCycles + id, (unsigned long long)(clock64() - tm));
      atomicAdd(p.mpCount + id, gn);  // groups evaluated
    }
  }
}

// ---- one stream group per item, resident exec levels -------------------------
// With one group per item (a single stream, or 8 streams per word and G = 1,
// e.g. thousands of queued streams of a small design) a warp has one word
// per lane and level, so a level is a chain of dependent shared-memory reads
// (unit range, unit word, header, lane record, operands, table) and
// instruction latencies, not throughput.  Resident level blocks do not change
// after the block set-up, so the first unit of a warp's NEXT level is read
// and decoded while the current level runs; after the level barrier only the
// operand loads, the lookup and the write-back are left.  A first unit that
// is not a one-level compact table record over a pool with slot immediates
// runs through the general unit path, as do a warp's further units.

// A word of a resident level block: the block never changes after the set-up
// (it is read only after the resident-copy wait, through addresses derived
// from its result), so the load is not volatile and the compiler may move it
// among the value-pool accesses.
__device__ __forceinline__ uint32_t ldsFixed(uint32_t a) {
  uint32_t v;
  asm("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(a));
  return v;
}

// Predicated accesses: no access where c is false.  ldsIf keeps `v` there;
// value-pool words are volatile as in ldsU32 / stsU32.
__device__ __forceinline__ uint32_t ldsIf(uint32_t a, bool c, uint32_t v) {
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q ld.shared.u32 %0, [%1];\n\t}"
               : "+r"(v)
               : "r"(a), "r"(uint32_t(c)));
  return v;
}
__device__ __forceinline__ uint2 ldsFixed2If(uint32_t a, bool c) {
  uint2 v = make_uint2(0u, 0u);
  asm("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %3, 0;\n\t@q ld.shared.v2.u32 {%0, %1}, [%2];\n\t}"
      : "+r"(v.x), "+r"(v.y)
      : "r"(a), "r"(uint32_t(c)));
  return v;
}
__device__ __forceinline__ void stsIf(uint32_t a, uint32_t v, bool c) {
  asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.shared.u32 [%0], %1;\n\t}" ::"r"(a), "r"(v),
               "r"(uint32_t(c))
               : "memory");
}

// A warp's part of one exec level, its first unit decoded.
struct WarpLevel1 {
  uint32_t ub, ue;    // the warp's units
  bool sync;          // the level starts with a block barrier
  bool simple;        // first unit: one-level compact LUT record, slot operands
  bool act, st;       // the lane evaluates a LUT / writes an entry back (simple only)
  uint32_t aA, aB, aC, lut, wA;  // operand and write-back slot addresses, lutIndex (0: pass c through)
};

// The words of level block blk a warp starts from: flags, unit range, and
// the first unit's record offset (the flags word when the warp has no unit,
// so every address stays inside the block).
struct WarpLevelHead {
  uint32_t flags, ub, ue, mp;
};

// Decodes the first unit of a warp's level (hdr: its header word).
__device__ __forceinline__ WarpLevel1 decodeWarpLevel1(const WarpLevelHead &h, uint32_t hdr, uint32_t vp,
                                                       uint32_t lane, bool constSlots) {
  WarpLevel1 r;
  r.sync = (h.flags & 1u) != 0u;
  r.ub = h.ub;
  r.ue = h.ue;
  const uint32_t W = (hdr >> 2) & 63u, nMid = (hdr >> 8) & 255u, nWB = (hdr >> 16) & 63u;
  r.simple = h.ub < h.ue && constSlots && (hdr & 3u) == kMPLut && (hdr & kMPCompact) != 0u &&
             (hdr & kMPFastTop) == 0u && nMid == 0u;
  r.act = r.simple && lane < W;
  r.st = r.simple && lane < nWB;
  // compact lane pair (as evalLutPass): a | b << 12 | (c & 255) << 24,
  // c >> 8 | write-back slot << 4 | lutIndex << 16; a lane without a LUT
  // (lane >= W) writes 0 to slot 0 when lane < nWB, as evalLutPass does
  const uint2 w = ldsFixed2If(h.mp + 4u * kMPHeaderWords + 8u * lane, r.act);
  r.lut = w.y >> 16;
  r.aA = vp + 4u * (w.x & 0xFFFu);
  r.aB = vp + 4u * ((w.x >> 12) & 0xFFFu);
  r.aC = vp + 4u * ((w.x >> 24) | ((w.y & 15u) << 8));
  r.wA = vp + 4u * ((w.y >> 4) & 0xFFFu);
  return r;
}

__device__ __forceinline__ WarpLevelHead readWarpLevelHead(uint32_t blk, uint32_t warp) {
  WarpLevelHead h;
  h.flags = ldsFixed(blk);
  h.ub = ldsFixed(blk + 4u * (1u + warp));
  h.ue = ldsFixed(blk + 4u * (2u + warp));
  h.mp = blk;
  return h;
}

// The record of a unit (hdr: its header word) decoded as decodeWarpLevel1
// does, for a level block staged or read from global memory.
template <bool SH>
__device__ __forceinline__ WarpLevel1 decodeUnit1(const Words<SH> mp, uint32_t hdr, uint32_t vp, uint32_t lane,
                                                  bool constSlots) {
  WarpLevel1 r;
  r.sync = false;
  r.ub = r.ue = 0u;
  const uint32_t W = (hdr >> 2) & 63u, nMid = (hdr >> 8) & 255u, nWB = (hdr >> 16) & 63u;
  r.simple = constSlots && (hdr & 3u) == kMPLut && (hdr & kMPCompact) != 0u && (hdr & kMPFastTop) == 0u &&
             nMid == 0u;
  r.act = r.simple && lane < W;
  r.st = r.simple && lane < nWB;
  const uint2 w = mp.at(kMPHeaderWords).pairIf(2u * lane, r.act);
  r.lut = w.y >> 16;
  r.aA = vp + 4u * (w.x & 0xFFFu);
  r.aB = vp + 4u * ((w.x >> 12) & 0xFFFu);
  r.aC = vp + 4u * ((w.x >> 24) | ((w.y & 15u) << 8));
  r.wA = vp + 4u * ((w.y >> 4) & 0xFFFu);
  return r;
}

template <int SPW, bool SH>
__device__ __forceinline__ void runUnitsOne(const KParams &p, const PartDesc &d, const Words<SH> blk,
                                            const Words<SH> units, uint32_t ub, uint32_t ue, uint32_t vp, uint32_t tab,
                                            uint32_t lane, uint32_t gb) {
  if (ub >= ue) return;
  const bool cs = p.constSlots != 0;
  WarpLevel1 now;
  {
    const Words<SH> mp = blk.at(units[ub] & kUnitOffsetMask);
    now = decodeUnit1<SH>(mp, mp[0], vp, lane, cs);
  }
  for (uint32_t u = ub; u < ue; ++u) {
    const bool more = u + 1 < ue;
    const uint32_t A = ldsIf(now.aA, now.act, 0u), B = ldsIf(now.aB, now.act, 0u), C = ldsIf(now.aC, now.act, 0u);
    // the next unit's record words go out beside this unit's operand loads
    // (records do not change during the level; a unit that reads what the
    // previous one wrote -- fused levels -- loads its operands after that
    // unit's write-back and warp barrier, in the next iteration)
    const uint32_t uw2 = more ? units[u + 1] : 0u;
    // inactive lanes: A = B = C = 0 and lut = 0, an address inside the table
    const uint32_t T = lookup<SPW>(tab, now.lut, A, B, C);
    const Words<SH> mp2 = blk.at(uw2 & kUnitOffsetMask);
    const uint32_t hdr2 = more ? mp2[0] : 0u;
    if (now.simple) {
      stsIf(now.wA, now.lut ? T : C, now.st);
      __syncwarp();
    } else {
      runUnit<SPW, 1, SH>(p, d, blk, units, u, vp, tab, lane, gb);
    }
    if (more) now = decodeUnit1<SH>(mp2, hdr2, vp, lane, cs);
  }
}

// Every exec level of one item of one stream group (G = 1), levels resident
// at res (the partition's first block at x0).  Same results as runLevel
// level by level.
// Per level the source order interleaves two dependent chains -- this
// level's operands, lookup and write-back, and the next level's unit range,
// unit word, header and lane record -- so that their shared-memory
// latencies overlap; the accesses are predicated instead of branched so the
// chains stay in one basic block.
template <int SPW>
__device__ __forceinline__ void runLevelsSingle(const KParams &p, const PartDesc &d, uint32_t res, uint32_t x0,
                                                const uint2 *__restrict__ ld, uint2 cur, uint2 nxt, uint32_t vp,
                                                uint32_t tab, uint32_t lane, uint32_t warp, uint32_t NW, uint32_t gb) {
  const bool cs = p.constSlots != 0;
  const uint2 zero2 = make_uint2(0u, 0u);
  WarpLevel1 now;
  {
    const uint32_t blk = res + 4u * (cur.x - x0);
    WarpLevelHead h = readWarpLevelHead(blk, warp);
    if (h.ub < h.ue) h.mp = blk + 4u * (ldsFixed(blk + 4u * (2u + NW + h.ub)) & kUnitOffsetMask);
    now = decodeWarpLevel1(h, ldsFixed(h.mp), vp, lane, cs);
  }
  for (uint32_t lv = 0; lv < d.nLevels; ++lv) {
    const uint2 after = lv + 2 < d.nLevels ? __ldg(ld + lv + 2) : zero2;
    const uint32_t blk = res + 4u * (cur.x - x0);
    // the next level's block (this one again after the last level: the
    // reads stay in bounds and their results are not used)
    const uint32_t nb = lv + 1 < d.nLevels ? res + 4u * (nxt.x - x0) : blk;
    if (lv > 0 && now.sync) __syncthreads();
    const uint32_t A = ldsIf(now.aA, now.act, 0u), B = ldsIf(now.aB, now.act, 0u), C = ldsIf(now.aC, now.act, 0u);
    WarpLevelHead h = readWarpLevelHead(nb, warp);
    const uint32_t uw = ldsFixed(h.ub < h.ue ? nb + 4u * (2u + NW + h.ub) : nb);
    // inactive lanes: A = B = C = 0 and lut = 0, an address inside the table
    const uint32_t T = lookup<SPW>(tab, now.lut, A, B, C);
    if (h.ub < h.ue) h.mp = nb + 4u * (uw & kUnitOffsetMask);
    const uint32_t hdr = ldsFixed(h.mp);
    stsIf(now.wA, now.lut ? T : C, now.st);
    __syncwarp();
    const WarpLevel1 next = decodeWarpLevel1(h, hdr, vp, lane, cs);
    for (uint32_t u = now.ub + (now.simple ? 1u : 0u); u < now.ue; ++u)
      runUnit<SPW, 1, true>(p, d, Words<true>{nullptr, blk}, Words<true>{nullptr, blk + 4u * (2u + NW)}, u, vp, tab,
                            lane, gb);
    now = next;
    cur = nxt;
    nxt = after;
  }
}

// ---- one partition for G groups (evalEachPartition, SimEval.cu:765-864) ---
// vp, tab: shared addresses of the block's value pool and truth table.
__device__ __forceinline__ PartDesc loadPart(const PartDesc *pd) {
  PartDesc d;
  const uint4 *src = reinterpret_cast<const uint4 *>(pd);
  uint4 *dst = reinterpret_cast<uint4 *>(&d);
#pragma unroll
  for (int i = 0; i < int(sizeof(PartDesc) / 16); ++i) dst[i] = __ldg(src + i);
  return d;
}

// Waits for the resident exec levels of the block (bulk copies on stage
// mbarrier 0, phase 0).  Bounded; false on a timeout.
__device__ bool residentWait(const KParams &p, uint32_t mb) {
  uint32_t done = 0;
  unsigned long long t0 = 0;
  for (uint32_t spin = 0; !done; ++spin) {
    asm volatile(
        "{\n\t.reg .pred P;\n\tmbarrier.try_wait.parity.shared::cta.b64 P, [%1], 0, %2;\n\tselp.u32 %0, 1, 0, P;\n\t}"
        : "=r"(done)
        : "r"(mb), "r"(kStageSuspendNs)
        : "memory");
    if (!done) {
      if (spin == 0) t0 = gtimer();
      else if (gtimer() - t0 > p.timeoutNs) {
        raiseErr(p, kErrTimeout, blockIdx.x, 0xFFFFFFFDu, 0);
        return false;
      }
    }
  }
  return true;
}

// res: shared address of the item's partition levels when they are resident
// (0: staged or read from global memory); resState: 0 levels not resident
// (or their copies timed out), 1 copies issued and not yet waited for, 2
// resident levels ready.
template <int SPW, int G, bool RES>
__device__ void evalItem(const KParams &p, uint32_t item, uint32_t vp, uint32_t tab, Stage &st, uint32_t cycle,
                         const uint32_t *retire, uint32_t res, uint32_t &resState) {
  const uint32_t pid = item & 0xFFFFFu, gb = item >> 20;
  // read-only loads: the descriptor stays valid across the shared-memory
  // stores (whose memory clobber would otherwise force global reloads)
  const PartDesc d = loadPart(p.parts + pid);
  const uint32_t tid = threadIdx.x, nthr = blockDim.x, lane = tid & 31u, warp = tid >> 5, NW = nthr >> 5;
  const uint2 *__restrict__ ld = p.levelDesc + d.schedOff;
  const uint32_t cap = p.stageWords;
  // level descriptors (block offset, words) are loaded two levels ahead so
  // their latency stays off the per-level path
  const uint2 zero2 = make_uint2(0u, 0u);
  uint2 cur = d.nLevels > 0 ? __ldg(ld) : zero2;
  uint2 nxt = d.nLevels > 1 ? __ldg(ld + 1) : zero2;
  const uint32_t x0 = cur.x;  // first level block of the partition (resident offset 0)
  // the first exec level streams in while the level-0 reads run
  // (the block's last warp issues the pieces: the other warps go straight
  // to their units instead of queueing copies behind the table lookups)
  if (cap && d.nLevels && cur.y <= cap && warp == NW - 1) stageCopy(st, 0, p.sched + cur.x, cur.y, lane, 32u);

  // level 0: register / exchange reads (evalPartL0RegRead / ExgRead)
  {
    const uint32_t n = d.l0Count;
    const uint32_t *src = p.net + d.l0Off;
    const uint32_t *dst = src + n;
    const uint32_t *pool = d.l0Exchange ? p.exg : p.regs;
    for (uint32_t i = tid; i < n; i += nthr) {
      const uint32_t s = __ldg(src + i);
      const uint32_t r = (__ldg(dst + (i >> 1)) >> ((i & 1u) * 16)) & 0xFFFFu;
      copyInG<G>(vpAddr<G>(vp, r, 0), pool + size_t(s) * p.gpad + gb * G);
    }
  }
  if (cap) stageCopyWait();  // the first level's pieces, before the barrier that publishes them
  __syncthreads();
  // resident levels: the block's copies were issued at setup and overlapped
  // the level-0 reads; on a (never expected) timeout the levels are read from
  // global memory and the error word ends the launch
  if constexpr (RES) {
    if (resState == 1u) resState = residentWait(p, st.mb0) ? 2u : 0u;
    if (resState != 2u) res = 0;
  }

  // exec levels: warp w runs the units the schedule gave it
  bool levelsDone = false;
  if constexpr (G == 1 && RES) {
    if (res && !(p.flags & kFlagProfileMP)) {
      runLevelsSingle<SPW>(p, d, res, x0, ld, cur, nxt, vp, tab, lane, warp, NW, gb);
      levelsDone = true;
    }
  }
  for (uint32_t lv = 0; lv < d.nLevels && !levelsDone; ++lv) {
    const uint2 after = lv + 2 < d.nLevels ? __ldg(ld + lv + 2) : zero2;
    bool staged = false;
    if constexpr (RES) {
      if (res) {
        const Words<true> blk{nullptr, res + 4u * (cur.x - x0)};
        if (lv > 0 && (blk[0] & 1u)) __syncthreads();
        runLevel<SPW, G, true>(p, d, blk, vp, tab, lane, warp, NW, gb);
        cur = nxt;
        nxt = after;
        continue;
      }
    }
    if (cap) {
      // level lv's pieces (copied during level lv - 1) are complete and, after
      // the barrier, visible; the buffers are reused every second level
      if (lv > 0) {
        stageCopyWait();
        __syncthreads();
      }
      if (lv + 1 < d.nLevels && nxt.y <= cap && warp == NW - 1)
        stageCopy(st, (lv + 1) & 1u, p.sched + nxt.x, nxt.y, lane, 32u);
      staged = cur.y <= cap;
    } else if (lv > 0 && (__ldg(p.sched + cur.x) & 1u)) {
      __syncthreads();
    }
    if (staged)
      runLevel<SPW, G, true>(p, d, Words<true>{nullptr, st.buf0 + (lv & 1u) * st.bytes}, vp, tab, lane, warp, NW, gb);
    else
      runLevel<SPW, G, false>(p, d, Words<false>{p.sched + cur.x, 0u}, vp, tab, lane, warp, NW, gb);
    cur = nxt;
    nxt = after;
  }
  __syncthreads();

  // signal capture: the value-pool slots the symbol file names as signals
  if (p.probeBuf)
    for (uint32_t i = tid; i < d.probeCount * G; i += nthr) {
      const uint32_t pi = i / G, g = i % G;
      const uint32_t slot = __ldg(p.net + d.probeOff + 2 * pi), idx = __ldg(p.net + d.probeOff + 2 * pi + 1);
      p.probeBuf[size_t(idx) * p.gpad + gb * G + g] = ldsU32(vpAddr<G>(vp, slot, g));
    }

  // last level (evalLastLevel / evalLastLevelExgWrite, SimEval.cu:625-761)
  // masks of streams retiring this cycle (admission): their registers take
  // the initial values, their memory writes / prints / stops are dropped
  uint32_t rm[G];
#pragma unroll
  for (int g = 0; g < G; ++g) rm[g] = retire ? __ldcg(retire + gb * G + g) : 0u;
  // stop exit: streams stopped in an earlier cycle keep their state; their
  // register words are rewritten with the values they hold (a stopped stream
  // that retires now takes the initial values instead)
  const bool stopExit = (p.flags & kFlagStopExit) != 0;
  uint32_t fm[G], xm[G];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    fm[g] = 0;
    if (stopExit) {
#pragma unroll
      for (int k = 0; k < SPW; ++k) {
        const uint32_t s = (gb * G + g) * SPW + k;
        if (s < p.nStreams && __ldcg(p.stopCycle + s) < cycle) fm[g] |= 15u << (4 * k);
      }
      fm[g] &= ~rm[g];
    }
    xm[g] = rm[g] | fm[g];  // streams whose writes are dropped this cycle
  }
  if (d.copyKind == 1 && (stopExit || retire)) {
    for (uint32_t i = tid; i < d.copySlots; i += nthr) {
      uint32_t init = 0;
      if (retire) {
        const uint32_t iv = p.initRegs[d.copyDst + i];
        init = SPW == 8 ? rep8(iv) : iv;
      }
      uint32_t *dst = p.regs + size_t(d.copyDst + i) * p.gpad + gb * G;
      uint32_t w[G];
      loadG<G>(vpAddr<G>(vp, d.copySrc + i, 0), w);
#pragma unroll
      for (int g = 0; g < G; ++g) {
        uint32_t v = (w[g] & ~xm[g]) | (init & rm[g]);
        if (stopExit) v |= __ldcg(dst + g) & fm[g];
        dst[g] = v;
      }
    }
  } else if (d.copyKind) {
    uint32_t *pool = d.copyKind == 1 ? p.regs : p.exg;
    for (uint32_t i = tid; i < d.copySlots; i += nthr)
      copyOutG<G>(pool + size_t(d.copyDst + i) * p.gpad + gb * G, vpAddr<G>(vp, d.copySrc + i, 0));
  }
  if (d.copyKind != 2) {
    for (uint32_t i = tid; i < d.memWCount * G; i += nthr) {
      const uint32_t opi = i / G, g = i % G;
      const uint32_t *r = p.net + d.memWOff + 4 * opi;
      const uint32_t lo = __ldg(r), hi = __ldg(r + 1), w2 = __ldg(r + 2), en = __ldg(r + 3);
      const unsigned long long memBase = (unsigned long long)lo | ((unsigned long long)(hi & 0x7FFFFFFFu) << 32);
      const bool multi = (hi >> 31) != 0;
      const uint32_t av = w2 & 0xFFFFu, dat = w2 >> 16;
      const uint32_t EN = (en < 16 ? rep8(en) : ldsU32(vpAddr<G>(vp, en, g))) & ~xm[g];
      const uint32_t DAT = dat < 16 ? rep8(dat) : ldsU32(vpAddr<G>(vp, dat, g));
      uint32_t AD[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) AD[j] = ldsU32(vpAddr<G>(vp, av + j, g));
#pragma unroll
      for (int k = 0; k < SPW; ++k) {
        const uint32_t s = (gb * G + g) * SPW + k;
        if (s >= p.nStreams || nib(EN, k) == 0) continue;
        uint32_t addr = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) addr |= nib(AD[j], k) << (4 * j);
        if (multi) addr <<= 2;
        const unsigned long long idx = memBase + addr;
        if (idx >= p.memPoolSize) {
          raiseErr(p, kErrMemRange, uint32_t(idx), uint32_t(idx >> 32), s);
          continue;
        }
        p.mems[s * p.memStride + idx] = uint8_t(nib(DAT, k));
      }
    }
    if (p.enablePrint) {
      for (uint32_t i = tid; i < d.printCount * G; i += nthr) {
        const uint32_t w = __ldg(p.net + d.printOff + i / G), g = i % G;
        const uint32_t en = w & 0xFFFFu, msg = w >> 16;
        const uint32_t EN = (en < 16 ? rep8(en) : ldsU32(vpAddr<G>(vp, en, g))) & ~xm[g];
        for (int k = 0; k < SPW; ++k) {
          const uint32_t s = (gb * G + g) * SPW + k;
          if (s < p.nStreams && nib(EN, k) != 0 && msg < p.nPrintMsgs) printf("%s", p.printMsgs[msg]);
        }
      }
    }
    for (uint32_t i = tid; i < d.stopCount * G; i += nthr) {
      const uint32_t opi = i / G, g = i % G;
      const uint32_t sw = __ldg(p.net + d.stopOff + opi), en = sw & 0xFFFFu;
      const uint32_t EN = (en < 16 ? rep8(en) : ldsU32(vpAddr<G>(vp, en, g))) & ~xm[g];
      for (int k = 0; k < SPW; ++k) {
        const uint32_t s = (gb * G + g) * SPW + k;
        if (s >= p.nStreams || nib(EN, k) == 0) continue;
        if (atomicExch(p.stop + s, 1u) == 0u) {
          p.stopCycle[s] = cycle;
          if (stopExit) {
            atomicAdd(p.nStopped, 1u);
            if (p.flags & kFlagSlots) p.eventHint[2u + (cycle & 1u)] = cycle + 1u;  // a retirement next cycle
          }
          if (p.printDiag) {
            printf("Toucan first stop: partition=%u op=%u enable_slot=%u value=%u\n", pid, opi, sw >> 16, nib(EN, k));
            for (uint32_t q = 0; q < d.printCount; ++q) {
              const uint32_t w = __ldg(p.net + d.printOff + q);
              if ((w & 0xFFFFu) == en && (w >> 16) < p.nPrintMsgs)
                printf("Stop-associated message (literal): %s\n", p.printMsgs[w >> 16]);
            }
          }
        }
      }
    }
  }
  // the next item reuses the value pool
  __syncthreads();
}

// ---- stimulus / digests ------------------------------------------------------
// Value of input `inp` of slot s for global cycle `cycle`; false when the slot
// takes no input that cycle (idle, past its stream's end, or a padding slot).
__device__ __forceinline__ bool stimValue(const KParams &p, uint32_t s, uint32_t cycle, uint32_t inp, uint32_t cur,
                                          uint32_t mask, uint32_t tog, uint32_t &v) {
  uint32_t lc;
  unsigned long long seed;
  if (s >= p.nStreams) return false;  // padding slot of the last group
  if ((p.flags & kFlagStopExit) && __ldcg(p.stopCycle + s) < cycle) return false;  // frozen after its stop
  if (p.flags & kFlagSlots) {
    const uint32_t q = __ldcg(p.slotStream + s);
    if (q == kNoStream || cycle >= __ldcg(p.slotRetire + s)) return false;
    lc = cycle - __ldcg(p.slotStart + s);
    seed = __ldg(p.jobSeed + q);
  } else {
    lc = cycle;
    seed = __ldg(p.streamSeed + s);
    if (p.stimTable) {
      v = __ldg(p.stimTable + (size_t(cycle - p.stimTableC0) * p.nStim + inp) * p.nStreams + s) & 15u;
      return true;
    }
  }
  const unsigned long long h = dmix64(seed ^ dmix64((unsigned long long)lc << 32 | inp));
  if (tog == 0)
    v = uint32_t(h) & mask;
  else
    v = (h >> 48) < tog ? cur ^ mask : cur;
  return true;
}

template <int SPW>
__device__ void applyStimulus(const KParams &p, uint32_t cycle, uint32_t gtid, uint32_t gthreads) {
  const uint32_t total = p.nStim * p.gpad;
  if constexpr (SPW == 8) {
    // eight lanes per register word, one stream each: the streams' slot
    // reads and hashes run side by side instead of one after another, and
    // the nibbles merge by shuffles within the lane octet.  Whole warps
    // iterate together (gthreads and the bound are multiples of 32).
    const uint32_t k = gtid & 7u, lanes = (total * 8u + 31u) & ~31u;
    for (uint32_t t = gtid; t < lanes; t += gthreads) {
      const uint32_t i = t >> 3;
      uint32_t part = 0, *wp = nullptr;
      if (i < total) {
        const uint32_t inp = i / p.gpad, g = i % p.gpad;
        const uint32_t reg = __ldg(p.stimReg + inp);
        const uint32_t mask = (1u << __ldg(p.stimBits + inp)) - 1u;
        const uint32_t tog = p.stimToggle ? uint32_t(__ldg(p.stimToggle + inp)) : 0u;
        wp = p.regs + size_t(reg) * p.gpad + g;
        const uint32_t cur = nib(__ldcg(wp), k);
        uint32_t v = cur;
        stimValue(p, g * SPW + k, cycle, inp, cur, mask, tog, v);
        part = v << (4u * k);
      }
      part |= __shfl_xor_sync(kFull, part, 1);
      part |= __shfl_xor_sync(kFull, part, 2);
      part |= __shfl_xor_sync(kFull, part, 4);
      if (wp && k == 0) *wp = part;
    }
  } else {
    // one stream per word
    for (uint32_t i = gtid; i < total; i += gthreads) {
      const uint32_t inp = i / p.gpad, g = i % p.gpad;
      const uint32_t reg = __ldg(p.stimReg + inp);
      const uint32_t mask = (1u << __ldg(p.stimBits + inp)) - 1u;
      const uint32_t tog = p.stimToggle ? uint32_t(__ldg(p.stimToggle + inp)) : 0u;
      uint32_t *wp = p.regs + size_t(reg) * p.gpad + g;
      const uint32_t cur = nib(__ldcg(wp), 0);
      uint32_t v = cur;
      stimValue(p, g, cycle, inp, cur, mask, tog, v);
      *wp = v;
    }
  }
}

// A slot retires in cycle t when its stream's last cycle was t - 1: the
// stream's length was reached, or (stop exit) it executed a stop op in t - 1.
__device__ __forceinline__ bool retiringAt(const KParams &p, uint32_t s, uint32_t t) {
  if (__ldcg(p.slotStream + s) == kNoStream) return false;
  if (__ldcg(p.slotRetire + s) == t) return true;
  if (!(p.flags & kFlagStopExit)) return false;
  const uint32_t sc = __ldcg(p.stopCycle + s);
  return sc != 0xFFFFFFFFu && sc + 1u == t;
}

// Streams whose register digest this cycle contributes: every active stream
// with per-cycle digests, else (admission) only the streams retiring now.
__device__ __forceinline__ bool digestStream(const KParams &p, uint32_t s, uint32_t cycle) {
  if (s >= p.nStreams) return false;
  if (p.flags & kFlagSlots) {
    if (__ldcg(p.slotStream + s) == kNoStream) return false;
    if (retiringAt(p, s, cycle)) return true;  // the retiring stream's final register digest
  }
  if ((p.flags & kFlagStopExit) && __ldcg(p.stopCycle + s) < cycle) return false;  // frozen
  return !(p.flags & kFlagSlots) || (p.flags & kFlagDigest);
}

// Per-cycle register digest: sum over i of mix64(i << 8 | nibble), per stream.
template <int SPW>
__device__ void digestSlice(const KParams &p, uint32_t cycle) {
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, NW = blockDim.x >> 5;
  const uint32_t chunks = (p.regSlots + 255) / 256;
  const uint32_t units = chunks * p.gpad;
  for (uint32_t u = blockIdx.x * NW + warp; u < units; u += p.nBlocks * NW) {
    const uint32_t g = u % p.gpad, ch = u / p.gpad;
    bool want[SPW];
    bool any = false;
#pragma unroll
    for (int k = 0; k < SPW; ++k) {
      want[k] = digestStream(p, g * SPW + k, cycle);
      any |= want[k];
    }
    if (!any) continue;
    unsigned long long acc[SPW];
#pragma unroll
    for (int k = 0; k < SPW; ++k) acc[k] = 0;
    const uint32_t end = min(p.regSlots, ch * 256 + 256);
    for (uint32_t i = ch * 256 + lane; i < end; i += 32) {
      const uint32_t w = __ldcg(p.regs + size_t(i) * p.gpad + g);
#pragma unroll
      for (int k = 0; k < SPW; ++k) acc[k] += dmix64((unsigned long long)i << 8 | nib(w, k));
    }
#pragma unroll
    for (int k = 0; k < SPW; ++k) {
      unsigned long long a = acc[k];
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
      if (lane == 0 && want[k]) atomicAdd(p.digAcc + g * SPW + k, a);
    }
  }
}

__device__ void foldDigest(const KParams &p, uint32_t cycle, uint32_t gtid, uint32_t gthreads) {
  for (uint32_t s = gtid; s < p.nStreams; s += gthreads) {
    uint32_t q = s, lc = cycle - p.cycBase;
    if ((p.flags & kFlagStopExit) && __ldcg(p.stopCycle + s) < cycle) continue;
    if (p.flags & kFlagSlots) {
      q = __ldcg(p.slotStream + s);
      if (q == kNoStream || retiringAt(p, s, cycle)) continue;  // retiring: kept for the admin phase
      lc = cycle - __ldcg(p.slotStart + s);
    }
    const unsigned long long dg = __ldcg(p.digAcc + s);
    p.digAcc[s] = 0;
    p.roll[s] = dmix64(p.roll[s] + dg);
    if (p.cycDig && lc < p.cycStride) p.cycDig[size_t(q) * p.cycStride + lc] = dg;
  }
}

// ---- admission events --------------------------------------------------------
// Retirements are found on the device: a stream may end at its length or, with
// stop exit, at its stop op, so no list is fixed in advance.  Queued streams
// are admitted in the order of queueOrder (longest first).
//
// A cycle is scanned only when a slot may retire in it.  eventHint words:
// [t & 1] a lower bound of the next length retirement as of cycle t (a scan
// in cycle t writes the bound for t + 1, admissions lower it; the graph form
// carries it from cycle to cycle, the persistent form keeps it in a register
// between scans); [2 + (c & 1)] = c + 1 when a stream stopped in cycle c.
// The words read in cycle t are written only in earlier cycles, so every block
// takes the same decision.
__device__ __forceinline__ bool mayRetire(const KParams &p, uint32_t t, uint32_t hint) {
  return t >= hint || ((p.flags & kFlagStopExit) && __ldcg(p.eventHint + 2u + ((t - 1u) & 1u)) == t);
}

// Every block builds the same bitmask of the slots retiring in cycle t (the
// state it reads was last written before this cycle's first region) and gets
// their number; block 0 writes the next length-retirement bound.
__device__ uint32_t scanRetiring(const KParams &p, uint32_t t, uint32_t *bits) {
  __shared__ uint32_t count, nextMin;
  const bool stopExit = (p.flags & kFlagStopExit) != 0;
  if (threadIdx.x == 0) {
    count = 0;
    nextMin = 0xFFFFFFFFu;
  }
  __syncthreads();
  const uint32_t nw = (p.nStreams + 31u) / 32u, lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  const uint32_t NW = blockDim.x >> 5;
  uint32_t c = 0, mn = 0xFFFFFFFFu;
  for (uint32_t w = warp; w < nw; w += NW) {
    const uint32_t s = w * 32u + lane;
    bool ret = false;
    if (s < p.nStreams) {
      const uint32_t q = __ldcg(p.slotStream + s), re = __ldcg(p.slotRetire + s), sc = __ldcg(p.stopCycle + s);
      if (q != kNoStream) {
        ret = re == t || (stopExit && sc != 0xFFFFFFFFu && sc + 1u == t);
        if (!ret) mn = min(mn, re);
      }
    }
    const uint32_t m = __ballot_sync(kFull, ret);
    if (lane == 0) {
      bits[w] = m;
      c += __popc(m);
    }
  }
  for (int o = 16; o > 0; o >>= 1) mn = min(mn, __shfl_xor_sync(kFull, mn, o));
  if (lane == 0) {
    if (c) atomicAdd(&count, c);
    if (blockIdx.x == 0) atomicMin(&nextMin, mn);
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0) p.eventHint[(t + 1u) & 1u] = nextMin;
  return count;
}

// The j-th set bit of the bitmask.
__device__ __forceinline__ uint32_t nthRetiring(const uint32_t *bits, uint32_t nw, uint32_t j) {
  for (uint32_t w = 0; w < nw; ++w) {
    uint32_t m = bits[w];
    const uint32_t c = __popc(m);
    if (j < c) {
      for (; j; --j) m &= m - 1u;
      return w * 32u + uint32_t(__ffs(int(m))) - 1u;
    }
    j -= c;
  }
  return 0xFFFFFFFFu;
}

// Region 0 of cycle t: list the retiring slots (block 0: the list, the count,
// the queue position and the retire masks) and digest their memories.
template <int SPW>
__device__ void eventRegion0(const KParams &p, const uint32_t *bits, uint32_t cnt) {
  const uint32_t nw = (p.nStreams + 31u) / 32u;
  if (blockIdx.x == 0) {
    if (threadIdx.x == 0) {
      *p.retCount = cnt;
      if (cnt) {
        uint32_t j = 0;
        for (uint32_t w = 0; w < nw; ++w)
          for (uint32_t m = bits[w]; m; m &= m - 1u) p.retList[j++] = w * 32u + uint32_t(__ffs(int(m))) - 1u;
        *p.queueSnap = __ldcg(p.queueHead);
      }
    }
    for (uint32_t j = threadIdx.x; j < cnt; j += blockDim.x) {
      const uint32_t s = nthRetiring(bits, nw, j);
      atomicOr(p.retireMask + s / SPW, 15u << (4 * (s % SPW)));
    }
  }
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5, NW = blockDim.x >> 5;
  const uint32_t chunk = 8192, chunks = (p.memPoolSize + chunk - 1) / chunk;
  const uint32_t units = cnt * chunks;
  for (uint32_t u = blockIdx.x * NW + warp; u < units; u += p.nBlocks * NW) {
    const uint32_t s = nthRetiring(bits, nw, u / chunks), ch = u % chunks;
    const uint8_t *m = p.mems + s * p.memStride;
    unsigned long long a = 0;
    const uint32_t end = min(p.memPoolSize, (ch + 1) * chunk);
    for (uint32_t i = ch * chunk + lane; i < end; i += 32) a += dmix64((unsigned long long)i << 8 | __ldcg(m + i));
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
    if (lane == 0) atomicAdd(p.memAcc + s, a);
  }
}

// Region 1 of a retire cycle: reset the retiring slots' memories (their
// memory writes are dropped this cycle).
__device__ void eventRegion1(const KParams &p, uint32_t gtid, uint32_t gthreads) {
  const uint32_t cnt = __ldcg(p.retCount);
  const uint32_t vecs = uint32_t((p.memPoolSize + 15ull) / 16);
  const size_t total = size_t(cnt) * vecs;
  for (size_t i = gtid; i < total; i += gthreads) {
    const uint32_t s = __ldcg(p.retList + uint32_t(i / vecs));
    const size_t v = i % vecs;
    reinterpret_cast<uint4 *>(p.mems + s * p.memStride)[v] = __ldg(reinterpret_cast<const uint4 *>(p.initMems) + v);
  }
}

// After the region-1 barrier: publish the retired streams' results and admit
// the next queued streams, in queue order, into the listed slots (with their
// cycle-0 inputs).
template <int SPW>
__device__ void eventAdmit(const KParams &p, uint32_t cycle, uint32_t gtid, uint32_t gthreads) {
  const uint32_t cnt = __ldcg(p.retCount), head = __ldcg(p.queueSnap);
  for (uint32_t j = gtid; j < cnt; j += gthreads) {
    const uint32_t s = __ldcg(p.retList + j);
    const uint32_t qn = head + j < p.nJobs ? __ldg(p.queueOrder + head + j) : kNoStream;
    const uint32_t q = __ldcg(p.slotStream + s), start = __ldcg(p.slotStart + s);
    p.outReg[q] = __ldcg(p.digAcc + s);
    p.outMem[q] = __ldcg(p.memAcc + s);
    p.outRoll[q] = __ldcg(p.roll + s);
    const uint32_t sc = __ldcg(p.stopCycle + s);
    p.outStop[q] = sc == 0xFFFFFFFFu ? sc : sc - start;
    atomicAdd(p.nDone, 1u);
    p.digAcc[s] = 0;
    p.memAcc[s] = 0;
    p.roll[s] = 0;
    p.stop[s] = 0;
    p.stopCycle[s] = 0xFFFFFFFFu;
    const uint32_t g = s / SPW, k = s % SPW;
    atomicAnd(p.retireMask + g, ~(15u << (4 * k)));
    if (qn == kNoStream) {
      p.slotStream[s] = kNoStream;
      continue;
    }
    p.slotStream[s] = qn;
    p.slotStart[s] = cycle + 1;
    p.slotRetire[s] = cycle + 1 + __ldg(p.jobLen + qn);
    atomicMin(p.eventHint + ((cycle + 1u) & 1u), cycle + 1 + __ldg(p.jobLen + qn));
    // primary inputs restart from the initial register values
    for (uint32_t inp = 0; inp < p.nStim; ++inp) {
      const uint32_t reg = __ldg(p.stimReg + inp);
      const uint32_t mask = (1u << __ldg(p.stimBits + inp)) - 1u;
      const uint32_t tog = p.stimToggle ? uint32_t(__ldg(p.stimToggle + inp)) : 0u;
      const uint32_t cur = p.initRegs[reg] & 15u;
      uint32_t v = cur;
      const unsigned long long h = dmix64(__ldg(p.jobSeed + qn) ^ dmix64((unsigned long long)0 << 32 | inp));
      if (tog == 0)
        v = uint32_t(h) & mask;
      else
        v = (h >> 48) < tog ? cur ^ mask : cur;
      uint32_t *wp = p.regs + size_t(reg) * p.gpad + g;
      atomicAnd(wp, ~(15u << (4 * k)));
      atomicOr(wp, v << (4 * k));
    }
  }
  if (gtid == 0) *p.queueHead = min(head + cnt, p.nJobs);
}

// ---- grid barrier (bounded) --------------------------------------------------
__device__ __forceinline__ bool gridSync(const KParams &p, uint32_t &gen) {
  __shared__ int ok;
  __syncthreads();
  // a one-block grid (a single stream of a small design): the block barrier
  // already orders the block's global writes before its later reads
  if (gridDim.x == 1) return true;
  if (threadIdx.x == 0) {
    ok = 1;
    // arrivals only ever add to the counter (zeroed before each launch):
    // barrier g of the launch is complete once it reaches g * blocks, so the
    // last block to arrive has nothing more to write (wrap-safe compare)
    const uint32_t target = (gen + 1u) * gridDim.x;
    __threadfence();
    const uint32_t arrived = atomicAdd(p.barrier, 1u) + 1u;
    if (arrived != target) {
      const unsigned long long t0 = gtimer();
      volatile uint32_t *vc = p.barrier;
      volatile uint32_t *ve = p.err;
      while (int32_t(*vc - target) < 0) {
        if (*ve != 0u) { ok = 0; break; }
        if (gtimer() - t0 > p.timeoutNs) {
          raiseErr(p, kErrTimeout, blockIdx.x, gen + 1u, 0);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    gen += 1u;
  }
  __syncthreads();
  return ok != 0;
}

// Stages the truth table into shared memory with one bulk async copy.
__device__ bool stageTable(const KParams &p, uint8_t *tab) {
  __shared__ __align__(8) unsigned long long mbar;
  const uint32_t mb = uint32_t(__cvta_generic_to_shared(&mbar));
  const uint32_t dst = uint32_t(__cvta_generic_to_shared(tab));
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(kLutTablePadded) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(p.lutTable), "r"(kLutTablePadded), "r"(mb)
                 : "memory");
  }
  uint32_t done = 0;
  const unsigned long long t0 = gtimer();
  while (!done) {
    asm volatile(
        "{\n\t.reg .pred P;\n\tmbarrier.try_wait.parity.shared::cta.b64 P, [%1], 0;\n\tselp.u32 %0, 1, 0, P;\n\t}"
        : "=r"(done)
        : "r"(mb)
        : "memory");
    if (!done && gtimer() - t0 > p.timeoutNs) {
      raiseErr(p, kErrTimeout, blockIdx.x, 0xFFFFFFFFu, 1);
      return false;
    }
  }
  return true;
}

// ---- kernels -----------------------------------------------------------------
// Shared-memory layout of a block: truth table, two exec-level stage buffers,
// value pool.  Returns false when staging the table timed out.
struct BlockSmem {
  uint32_t tab;  // shared address of the truth table
  uint32_t vp;   // shared address of the value pool
  uint32_t res;  // shared address of the resident exec levels
  uint32_t resState;  // see evalItem
  Stage st;
};

// region: the region whose resident levels are loaded (-1: both, for the
// persistent form).  With resident levels, stage mbarrier 0 (no stage
// buffers then) completes their copies.
template <int G, bool RES>
__device__ __forceinline__ bool setupBlock(const KParams &p, uint8_t *smem, unsigned long long *stageMbar, BlockSmem &b,
                                           int region) {
  const uint32_t base = uint32_t(__cvta_generic_to_shared(smem));
  b.tab = base;
  b.st.buf0 = base + kLutTablePadded;
  b.st.bytes = p.stageWords * 4u;
  b.st.mb0 = uint32_t(__cvta_generic_to_shared(&stageMbar[0]));
  b.res = b.st.buf0 + 2u * b.st.bytes;
  b.vp = b.res + (RES ? 4u * p.resWords : 0u);
  b.resState = 0;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b.st.mb0) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b.st.mb0 + 8u) : "memory");
  }
  if (p.constSlots)  // immediates 0..15 in value-pool slots 0..15
    for (uint32_t i = threadIdx.x; i < 16u * G; i += blockDim.x) stsU32(b.vp + 4u * i, rep8(i / G));
  const bool staged = stageTable(p, smem);
  __syncthreads();
  if (RES && p.resWords) {
    // the block's partitions: one bulk copy each, completed on mbarrier 0
    const uint32_t r0 = region < 0 ? 0u : uint32_t(region), r1 = region < 0 ? 1u : uint32_t(region);
    uint32_t n = 0;
    for (uint32_t r = r0; r <= r1; ++r) {
      const uint32_t *cb = p.resCopyBegin + r * (p.nBlocks + 1);
      n += __ldg(cb + blockIdx.x + 1) - __ldg(cb + blockIdx.x);
    }
    if (n) {
      b.resState = 1;
      if (threadIdx.x == 0) {
        uint32_t bytes = 0;
        for (uint32_t r = r0; r <= r1; ++r) {
          const uint32_t *cb = p.resCopyBegin + r * (p.nBlocks + 1);
          for (uint32_t c = __ldg(cb + blockIdx.x); c < __ldg(cb + blockIdx.x + 1); ++c) bytes += 4u * __ldg(p.resCopy + 3 * c + 1);
        }
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b.st.mb0), "r"(bytes) : "memory");
        for (uint32_t r = r0; r <= r1; ++r) {
          const uint32_t *cb = p.resCopyBegin + r * (p.nBlocks + 1);
          for (uint32_t c = __ldg(cb + blockIdx.x); c < __ldg(cb + blockIdx.x + 1); ++c) {
            const uint32_t src = __ldg(p.resCopy + 3 * c), words = __ldg(p.resCopy + 3 * c + 1);
            const uint32_t dst = b.res + 4u * __ldg(p.resCopy + 3 * c + 2);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                "l"(p.sched + src), "r"(4u * words), "r"(b.st.mb0)
                : "memory");
          }
        }
      }
    }
  }
  return staged;
}

// One region of cycle t for this block: its items, then the region's side
// work (digests and retiring-stream capture in region 0; memory reset of
// retiring streams, next cycle's inputs and digest folding in region 1).
template <int SPW, int G, bool RES>
__device__ void regionWork(const KParams &p, BlockSmem &b, uint32_t t, uint32_t r, bool event, const uint32_t *retBits,
                           uint32_t retCnt, uint32_t cEnd, uint32_t c0) {
  const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gthreads = p.nBlocks * blockDim.x;
  const uint32_t *ib = p.itemBegin + r * (p.nBlocks + 1);
  const uint32_t i0 = __ldg(ib + blockIdx.x), i1 = __ldg(ib + blockIdx.x + 1);
  for (uint32_t i = i0; i < i1; ++i) {
    const long long tk = clock64();
    const uint32_t item = __ldg(p.items + i);
    const uint32_t res = RES && p.resWords ? b.res + 4u * __ldg(p.itemRes + i) : 0u;
    evalItem<SPW, G, RES>(p, item, b.vp, b.tab, b.st, t, (event && r == 1) ? p.retireMask : nullptr, res, b.resState);
    // per-partition clock64 profile (SimEval.cu:894-983): running mean of the
    // useful ticks over cycles [100, 200) of a launch, group block 0
    if ((p.flags & kFlagProfile) && threadIdx.x == 0 && (item >> 20) == 0 && t >= c0 + 100 && t < c0 + 200) {
      const uint32_t pid = item & 0xFFFFFu, pc = t - c0 - 100;
      p.profUseful[pid] = (p.profUseful[pid] * pc + (clock64() - tk)) / (pc + 1);
    }
  }
  if (r == 0) {
    if ((p.flags & kFlagDigest) || event) digestSlice<SPW>(p, t);
    if (p.flags & kFlagSlots) eventRegion0<SPW>(p, retBits, retCnt);  // the cycle's list, also when empty
  } else {
    if (event) eventRegion1(p, gtid, gthreads);
    // (stop exit: applied after the region barrier, when every stop of the cycle is known)
    if ((p.flags & kFlagStimulus) && !(p.flags & kFlagStopExit) && t + 1 < cEnd) applyStimulus<SPW>(p, t + 1, gtid, gthreads);
    if (p.flags & kFlagDigest) foldDigest(p, t, gtid, gthreads);
  }
}

// Persistent form: every cycle of the launch, regions separated by the
// bounded grid barrier.  Per cycle: region 0, region 1, (stop exit) the next
// cycle's inputs, (a retirement) admission; the launch ends early once every
// queued stream retired or, resident streams with stop exit, every stream
// stopped.
template <int SPW, int G, bool RES>
__global__ void __launch_bounds__(1024) cycleKernel(const KParams p, uint32_t c0, uint32_t nCycles) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) unsigned long long stageMbar[2];
  __shared__ uint32_t retBits[kMaxSlotWords];
  BlockSmem b;
  if (!setupBlock<G, RES>(p, smem, stageMbar, b, -1)) return;
  const uint32_t gtid = blockIdx.x * blockDim.x + threadIdx.x, gthreads = p.nBlocks * blockDim.x;
  const uint32_t cEnd = c0 + nCycles;
  uint32_t gen = 0;
  if (p.flags & kFlagStimulus) {
    applyStimulus<SPW>(p, c0, gtid, gthreads);
    if (!gridSync(p, gen)) return;
  }
  const bool slots = (p.flags & kFlagSlots) != 0;
  uint32_t hint = slots ? __ldcg(p.eventHint + (c0 & 1u)) : 0xFFFFFFFFu;
  for (uint32_t t = c0; t < cEnd; ++t) {
    const bool scan = slots && mayRetire(p, t, hint);  // the same in every block
    const uint32_t retCnt = scan ? scanRetiring(p, t, retBits) : 0u;
    const bool event = retCnt > 0;
#pragma unroll 1
    for (uint32_t r = 0; r < 2; ++r) {
      const long long tStart = clock64();
      regionWork<SPW, G, RES>(p, b, t, r, event, retBits, retCnt, cEnd, c0);
      if (!gridSync(p, gen)) return;
      if ((p.flags & kFlagProfile) && threadIdx.x == 0 && t >= c0 + 100 && t < c0 + 200) {
        const long long total = clock64() - tStart;
        const uint32_t pc = t - c0 - 100;
        const uint32_t *ib = p.itemBegin + r * (p.nBlocks + 1);
        for (uint32_t i = __ldg(ib + blockIdx.x); i < __ldg(ib + blockIdx.x + 1); ++i) {
          const uint32_t item = __ldg(p.items + i);
          if ((item >> 20) != 0) continue;
          const uint32_t pid = item & 0xFFFFFu;
          p.profTotal[pid] = (p.profTotal[pid] * pc + total) / (pc + 1);
        }
      }
    }
    if ((p.flags & kFlagStopExit) && (p.flags & kFlagStimulus) && t + 1 < cEnd) {
      applyStimulus<SPW>(p, t + 1, gtid, gthreads);
      if (!gridSync(p, gen)) return;
    }
    if (event) {
      eventAdmit<SPW>(p, t, gtid, gthreads);
      if (!gridSync(p, gen)) return;
    }
    if ((p.flags & kFlagCountCycles) && blockIdx.x == 0 && threadIdx.x == 0) *p.realCycles += 1;
    // every block reads the words after the cycle's last barrier: same decision
    if (scan) {
      hint = __ldcg(p.eventHint + ((t + 1u) & 1u));  // this scan's bound, lowered by the admissions
      if (__ldcg(p.nDone) >= p.nJobs) break;
    } else if (!slots && (p.flags & kFlagStopExit) && __ldcg(p.nStopped) >= p.nStreams) {
      break;
    }
  }
}

// Graph form: one launch per region, kernel boundaries instead of the grid
// barrier; cycle = device counter + k so one captured chunk is replayed.
template <int SPW, int G, bool RES>
__global__ void __launch_bounds__(1024) regionKernel(const KParams p, uint32_t k, uint32_t r) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) unsigned long long stageMbar[2];
  __shared__ uint32_t retBits[kMaxSlotWords];
  // graph state and the error word are written only by earlier launches
  const uint32_t t = __ldcg(p.graphState) + k, cEnd = __ldcg(p.graphState + 2);
  if (t >= cEnd || __ldcg(p.graphState + 4) || __ldcg(p.err)) return;
  const bool slots = (p.flags & kFlagSlots) != 0;
  // admission words, loaded before the block setup hides their latency
  const uint32_t adm = !slots ? 0u : r == 0 ? __ldcg(p.eventHint + (t & 1u)) : __ldcg(p.retCount);
  BlockSmem b;
  if (!setupBlock<G, RES>(p, smem, stageMbar, b, int(r))) return;
  uint32_t retCnt = adm;
  if (slots && r == 0) {
    retCnt = 0;
    if (mayRetire(p, t, adm))
      retCnt = scanRetiring(p, t, retBits);
    else if (blockIdx.x == 0 && threadIdx.x == 0)
      p.eventHint[(t + 1u) & 1u] = adm;  // carried to the next cycle's launch
  }
  regionWork<SPW, G, RES>(p, b, t, r, retCnt > 0, retBits, retCnt, cEnd, __ldcg(p.graphState + 3));
}

// Kernel pointers by (streams per word, groups per item) for one exec-level
// source (RES: resident for the launch; else staged per level or global);
// each instantiating translation unit takes one form and one RES.
template <bool RES>
void *cycleKernelPtrT(int spw, int G) {
  if (spw == 1) return reinterpret_cast<void *>(&cycleKernel<1, 1, RES>);
  if (G == 8) return reinterpret_cast<void *>(&cycleKernel<8, 8, RES>);
  if (G == 4) return reinterpret_cast<void *>(&cycleKernel<8, 4, RES>);
  if (G == 2) return reinterpret_cast<void *>(&cycleKernel<8, 2, RES>);
  return reinterpret_cast<void *>(&cycleKernel<8, 1, RES>);
}

template <bool RES>
void *regionKernelPtrT(int spw, int G) {
  if (spw == 1) return reinterpret_cast<void *>(&regionKernel<1, 1, RES>);
  if (G == 8) return reinterpret_cast<void *>(&regionKernel<8, 8, RES>);
  if (G == 4) return reinterpret_cast<void *>(&regionKernel<8, 4, RES>);
  if (G == 2) return reinterpret_cast<void *>(&regionKernel<8, 2, RES>);
  return reinterpret_cast<void *>(&regionKernel<8, 1, RES>);
}

}  // namespace
}  // namespace tgs
