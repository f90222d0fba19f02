// Batched search kernel with a decoupled staging pipeline (sm_103a).
//
// The same work and arithmetic as the fast form of semb_search_kernel (FP16/BF16
// store, sample-unit traveltimes, Kahan energy, top-4 per (CDP, t0)), but the
// warps of a CTA no longer meet at a CTA-wide barrier twice per chunk.  Chunks
// of aperture traces flow through a ring:
//
//   one warp plans chunk c+2 and starts its TMA copies into raw buffer (c+2) % 2
//   every warp converts its share of chunk c+1 into quad stage (c+1) % 3
//   every warp computes chunk c from quad stage c % 3
//
// Hand-offs are mbarriers: raw_full (TMA bytes landed), q_full (every warp has
// converted its share of a chunk) and q_empty (every warp has computed a chunk).
// A warp may run a whole chunk ahead of the slowest one, which absorbs the
// scheduling skew that a CTA barrier turns into idle warps.  The extra duties
// rotate so that no warp is systematically behind: chunk c is planned by warp
// c % nwarps (the planner of chunk c-1 has finished: its copies' barrier, which
// every warp has seen complete before planning, is armed at the end of planning)
// and the conversion of chunk c starts its round-robin at that warp too.  The
// chunk stream is flat across passes and tasks: the planner fetches tasks from
// the work queue and tags each chunk with its task, pass and first/last flags; the
// warp that finalizes a task last merges every warp's top-4 lists (no CTA barrier
// there either).
//
// Every wait is bounded (kWaitNs on %globaltimer).  A warp that gives up sets
// ST_TIMEOUT and leaves; the others then give up at their next wait, each first
// waiting (bounded) for the copies still in flight.
#pragma once

#include "semb_kernels.cuh"

namespace semb {

constexpr int kStages = 3;     // quad stages
constexpr int kMetaRing = 4;   // chunk metadata and copy descriptors
constexpr int kRawBufs = 2;    // raw (TMA) buffers

enum : int { CH_PASS_FIRST = 1, CH_PASS_LAST = 2, CH_TASK_LAST = 4, CH_END = 8 };

// Chunk tags written by the planner next to the chunk metadata.
struct ChunkTag {
  int flags;
  int cdp;
  int t0s;
  int pass;
  int napert;
  int ic_lo;   // Z0: the pass's first C index
  int zslot;   // Z0: the pass slot of its central traces' sums
  int pad;
};

// The planners' position in the chunk stream.
struct Producer {
  int64_t pos, begin, end;
  int task;   // -1: fetch the next task
  int cdp, t0s, pass;
  int done;   // the end-of-stream chunk has been issued
  int next;   // index of the next chunk to produce
  float T_lo, T_hi;
  int64_t zb, ze;   // Z0: the task's central traces (entries zb .. ze-1)
  int64_t zpos;     // Z0: the next central trace to add to the pass's sums
  int pseq;         // Z0: passes started; the pass slot is pseq % kZ0Slots
  int zslot, ic_lo; // Z0: the current pass's slot and first C index
};

// Shared-memory layout (bytes), shared by host and device:
//   [0, 128)   mbarriers (raw_full[2], q_full[3], q_empty[3], merge_done) and the
//              merge counter
//   prod       producer state
//   meta[4]    chunk metadata, tag[4] chunk tags
//   src[4]     copy descriptors
//   tops       running top-4 per thread [3][4][NT]
//   kahan      Kahan totals and compensations [2][RC][NT]
//   quad[3]    staged 16-byte entries, each followed by its zero block
//   raw[2]     raw windows (TMA destination)
//   z0         Z0 variants: the central traces' sums of the passes in flight,
//              [kZ0Slots][kZ0C][5][32] floats
struct PipeLayout {
  size_t prod, meta, tag, src, z0, tops, kahan, quad, quad_stride, raw, raw_stride, total;
};

constexpr size_t kZ0SlotFloats = (size_t)kZ0C * 5 * 32;

__host__ __device__ inline PipeLayout pipe_layout(int rc, int cap, int storage, int nt, int lay, int z0 = 0) {
  PipeLayout L;
  L.prod = 128;
  L.meta = L.prod + align128(sizeof(Producer));
  L.tag = L.meta + kMetaRing * kMetaBytes;
  L.src = L.tag + align128(kMetaRing * sizeof(ChunkTag));
  L.z0 = L.src + (size_t)kMetaRing * kMaxChunk * 16;
  L.tops = L.z0 + (z0 ? (size_t)kZ0Slots * kZ0SlotFloats * 4 : 0);
  L.kahan = L.tops + align128(3 * (size_t)kTopK * nt * 4);
  L.quad = L.kahan + align128(2 * (size_t)rc * nt * 4);
  // LAY_X3: a sample plane and a difference plane of kXPlane floats each (the plan
  // keeps cap + kZeroSlots within a plane)
  L.quad_stride = lay == LAY_X3 ? (size_t)8 * kXPlane : align128(((size_t)cap + kZeroSlots) * lay_stage_bytes(lay));
  L.raw = L.quad + kStages * L.quad_stride;
  L.raw_stride = align128(((size_t)cap + 8 * kMaxChunk) * (storage == STORE_F32 ? 4 : 2));
  L.total = L.raw + kRawBufs * L.raw_stride;
  return L;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Z0 (CRS, w = 3): the sums of a task's central traces at zero midpoint distance,
// which every (A, B) of one C shares: with |dm| = 0 an item's traveltime is
// t^2 = fma(t0, t0, C h) whatever A and B.  Computed with the items' own FP32
// operations (the traveltime, its sample index and weight, and the interpolation of the
// packed value/difference staging), so each trace adds what it would add to every
// item of that C.  Adds central traces kb .. ke-1 (of the task's zb .. ze-1) to the
// pass slot: one lane per t0 of the task (lane = t0 - t0s), C indices c_lo ..
// c_lo + nc - 1; slot[(ci * 5 + q) * 32 + lane] holds the three window numerators, the
// energy and the count of in-range traces (as a float).  Samples are read from the
// trace store in global memory, within each trace's row (an in-range window ends at
// most two samples past the record, inside the row's zero padding); a CDP's own traces
// are consecutive in the store and in its aperture list.
static __device__ __noinline__ void central_add(const KParams& P, int t0s, int64_t zb, int64_t kb, int64_t ke,
                                                int c_lo, int nc, float* slot) {
  const int lane = threadIdx.x & 31;
  const float T = (float)min(t0s + lane, P.ns - 1);
  const unsigned span = (unsigned)(P.ns - 2 * P.tau - 2);
  const int tr0 = kb < ke ? __ldg(P.ap_tr + zb) : 0;
  for (int ci = 0; ci < nc; ++ci) {
    const float cc = P.cvals[c_lo + ci];
    float* z = slot + ci * 5 * 32 + lane;
    float n0 = z[0], n1 = z[32], n2 = z[64], den = z[96], m = z[128];
    for (int64_t k = kb; k < ke; ++k) {
      const float4 g = __ldg(P.ap_geo + k);
      if (g.x != 0.f) continue;
      const float t = sqrt_fast(fmaf(T, T, cc * g.z));
      const float y = __fadd_rz(t, 8388608.0f);
      const int rel = __float_as_int(y) - (0x4B000000 + P.tau);   // it - tau
      if ((unsigned)rel > span) continue;
      const float x = t - (y - 8388608.0f);
      const int tr = tr0 + (int)(k - zb);
      const int64_t at = (int64_t)tr * P.pitch + rel;
      float v[4];
      if (P.storage == STORE_F32) {
#pragma unroll
        for (int u = 0; u < 4; ++u) v[u] = __ldg(P.samples + at + u);
      } else {
        const float sc = __ldg(P.scale + tr);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const uint32_t b = __ldg(P.samples16 + at + u);
          v[u] = (P.storage == STORE_F16 ? half_bits_to_float(b) : __uint_as_float(b << 16)) * sc;
        }
      }
      // the packed value/difference entry (s_0, s_2, d_0, d_2) and its window
      const float d0 = v[1] - v[0], d2 = v[3] - v[2];
      const float w0 = fmaf(d0, x, v[0]), w2 = fmaf(d2, x, v[2]);
      const float s1 = v[0] + d0;
      const float w1 = fmaf(v[2] - s1, x, s1);
      n0 += w0;
      n1 += w1;
      n2 += w2;
      den = fmaf(w0, w0, den);
      den = fmaf(w1, w1, den);
      den = fmaf(w2, w2, den);
      m += 1.f;
    }
    z[0] = n0;
    z[32] = n1;
    z[64] = n2;
    z[96] = den;
    z[128] = m;
  }
}

// TU: unroll factor of the in-range trace loop (independent work of TU traces in
// flight per iteration).
// GLOB: as for semb_search_kernel, the variant may stage less than a whole trace.
// Z0 > 0 (CRS B-run, packed value/difference staging): the planner leaves the task's
// central traces at zero midpoint distance out of the chunks and adds their sums for
// each C index of the pass into the pass's slot, Z0 traces with each chunk it plans and
// the rest with the pass's last (central_add); each item adds those of its C when it
// finalizes the pass.
template <int METHOD, int W, int RC, int MINB, int LAY, bool BRUN, int NT, int TU = 1, bool GLOB = false,
          int Z0 = 0>
__global__ void __launch_bounds__(NT, MINB) semb_pipe_kernel(KParams P) {
  static_assert(!Z0 || (METHOD == METHOD_CRS && BRUN && W == 3 && stage_lay(LAY) == LAY_PD),
                "central-trace sharing is for the CRS B-run packed value/difference kernel");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const PipeLayout L = pipe_layout(RC, P.cap, P.storage, NT, LAY, Z0 ? 1 : 0);
  float* z0_base = reinterpret_cast<float*>(smem_raw + L.z0);
  auto z0_slot = [&](int slot) { return z0_base + (size_t)slot * kZ0SlotFloats; };
  constexpr uint32_t EB = lay_entry_bytes(LAY);   // bytes per staged entry
  uint64_t* raw_full = reinterpret_cast<uint64_t*>(smem_raw);   // [kRawBufs]
  uint64_t* q_full = raw_full + kRawBufs;                        // [kStages]
  uint64_t* q_empty = q_full + kStages;                          // [kStages]
  uint64_t* merge_done = q_empty + kStages;                      // [1]
  int* merge_cnt = reinterpret_cast<int*>(smem_raw + 96);
  Producer* prod = reinterpret_cast<Producer*>(smem_raw + L.prod);
  auto meta_at = [&](int c) {
    return reinterpret_cast<ChunkMeta*>(smem_raw + L.meta + (size_t)(c % kMetaRing) * kMetaBytes);
  };
  auto tag_at = [&](int c) { return reinterpret_cast<ChunkTag*>(smem_raw + L.tag) + (c % kMetaRing); };
  auto src_at = [&](int c) { return reinterpret_cast<int4*>(smem_raw + L.src) + (c % kMetaRing) * kMaxChunk; };
  auto quad_at = [&](int c) {
    return reinterpret_cast<float4*>(smem_raw + L.quad + (size_t)(c % kStages) * L.quad_stride);
  };
  auto raw_at = [&](int c) { return smem_raw + L.raw + (size_t)(c % kRawBufs) * L.raw_stride; };
  constexpr int K = kTopK;
  float* top_s = reinterpret_cast<float*>(smem_raw + L.tops);   // [K][NT]
  int* top_i = reinterpret_cast<int*>(top_s + K * NT);
  float* top_k = top_s + 2 * K * NT;
  float* kahan_hi = reinterpret_cast<float*>(smem_raw + L.kahan);   // [RC][NT]
  float* kahan_lo = kahan_hi + RC * NT;

  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  constexpr float kSent = (METHOD == METHOD_CMP) ? -1.0f : 0.0f;

  for (int s = 0; s < kStages; ++s) {
    if (threadIdx.x < kZeroSlots * (EB / 16))
      quad_at(s)[P.cap * (EB / 16) + threadIdx.x] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (LAY == LAY_X3 && threadIdx.x < kZeroSlots) {   // both planes' zero blocks
      reinterpret_cast<float*>(quad_at(s))[P.cap + threadIdx.x] = 0.f;
      reinterpret_cast<float*>(quad_at(s))[kXPlane + P.cap + threadIdx.x] = 0.f;
    }
    if (LAY == LAY_FT && threadIdx.x < kZeroSlots)   // the side entries' zero block
      reinterpret_cast<float2*>(quad_at(s) + P.cap + kZeroSlots)[P.cap + threadIdx.x] = make_float2(0.f, 0.f);
  }
  if (threadIdx.x == 0) {
    for (int b = 0; b < kRawBufs; ++b) mbar_init(&raw_full[b], 1);
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&q_full[s], nwarps);
      mbar_init(&q_empty[s], nwarps);
    }
    mbar_init(merge_done, 1);
    *merge_cnt = 0;
    prod->task = -1;
    prod->done = 0;
    prod->pseq = 0;
    prod->zslot = prod->ic_lo = 0;
    prod->zpos = 0;
    prod->next = 0;
    fence_mbar_init();
  }
  __syncthreads();

  // the planner warp: plan the next chunk of the stream and start its copies
  auto produce = [&]() {
    const int c = prod->next;
    ChunkMeta* m = meta_at(c);
    ChunkTag* tg = tag_at(c);
    int4* src = src_at(c);
    if (prod->task < 0) {
      int t = 0;
      if (lane == 0) t = atomicAdd(P.counter, 1);
      t = __shfl_sync(0xffffffffu, t, 0);
      __syncwarp();
      if (t >= P.ntasks) {
        if (lane == 0) {
          m->n = 0;
          m->n_in = 0;
          m->consumed = 0;
          m->bytes = 0;
          tg->flags = CH_END;
          prod->done = 1;
          prod->next = c + 1;
        }
        __syncwarp();
        issue_raw(P, m, src, raw_at(c), &raw_full[c % kRawBufs]);
        return;
      }
      const int2 td = P.tasks[t];
      if (lane == 0) {
        prod->task = t;
        prod->cdp = td.x;
        prod->t0s = td.y;
        prod->begin = P.ap_off[td.x];
        prod->end = P.ap_off[td.x + 1];
        prod->pos = prod->begin;
        prod->pass = 0;
        prod->T_lo = P.dt * (float)td.y;
        prod->T_hi = P.dt * (float)min(td.y + kTB - 1, P.ns - 1);
        prod->zb = prod->ze = 0;
        if (Z0) {
          const int2 zr = P.z0r[td.x];
          prod->zb = prod->begin + zr.x;
          prod->ze = prod->zb + zr.y;
        }
      }
      __syncwarp();
    }
    const int64_t pos = prod->pos, begin = prod->begin, end = prod->end;
    const int pass = prod->pass;
    int flags = pos == begin ? CH_PASS_FIRST : 0;
    plan_chunk<METHOD, FORM_FAST>(P, P.pass_bounds + pass * 8, pos, end, prod->T_lo, prod->T_hi, m, src, prod->zb,
                                  prod->ze);
    const int64_t npos = pos + m->consumed;
    if (Z0) {
      // the central traces' sums of the pass: a new pass takes the next slot, zeroed;
      // each chunk adds the next Z0 traces, the pass's last chunk all the rest
      const int2 pc = P.pass_c[pass];
      const int slot = pos == begin ? prod->pseq % kZ0Slots : prod->zslot;
      float* zs = z0_slot(slot);
      int64_t kb = prod->zpos;
      if (pos == begin) {
        kb = prod->zb;
        for (int q = lane; q < (int)kZ0SlotFloats; q += 32) zs[q] = 0.f;
      }
      const int64_t ke = npos >= end ? prod->ze : min(prod->ze, kb + (int64_t)Z0);
      __syncwarp();
      central_add(P, prod->t0s, prod->zb, kb, ke, pc.x, pc.y, zs);
      __syncwarp();
      if (lane == 0) {
        if (pos == begin) prod->pseq += 1;
        prod->zslot = slot;
        prod->ic_lo = pc.x;
        prod->zpos = ke;
        tg->zslot = slot;
        tg->ic_lo = pc.x;
      }
    }
    if (lane == 0) {
      if (npos >= end) {
        flags |= CH_PASS_LAST;
        prod->pos = begin;
        prod->pass = pass + 1;
        if (pass + 1 == P.npass) {
          flags |= CH_TASK_LAST;
          prod->task = -1;
        }
      } else {
        prod->pos = npos;
      }
      tg->flags = flags;
      tg->cdp = prod->cdp;
      tg->t0s = prod->t0s;
      tg->pass = pass;
      tg->napert = (int)(end - begin);
      prod->next = c + 1;
    }
    __syncwarp();
    issue_raw(P, m, src, raw_at(c), &raw_full[c % kRawBufs]);
  };

  int raw_seen = 0;   // chunks whose raw barrier this thread has seen complete
  // a bounded wait failed: report it and wait (bounded) for the copies in flight
  auto give_up = [&]() {
    if (lane == 0) atomicOr(P.status, ST_TIMEOUT);
    const int issued = min(prod->next, raw_seen + kRawBufs);
    for (int c = raw_seen; c < issued; ++c) wait_bar(&raw_full[c % kRawBufs], (c / kRawBufs) & 1);
  };

  // every warp: convert its share of chunk c into quad stage c % kStages
  auto convert_step = [&](int c) -> bool {
    if (c >= kStages && !wait_bar(&q_empty[c % kStages], (c / kStages - 1) & 1)) return false;
    if (!wait_bar(&raw_full[c % kRawBufs], (c / kRawBufs) & 1)) return false;
    raw_seen = c + 1;
    convert_chunk<LAY>(P, meta_at(c), src_at(c), raw_at(c), quad_at(c), c % nwarps);
    __syncwarp();
    if (lane == 0) mbar_arrive(&q_full[c % kStages]);
    return true;
  };

  // chunks 0 and 1 (warp 0; the copies' barrier of chunk 0 orders them for the
  // planner of chunk 2)
  if (warp == 0) {
    produce();
    if (!prod->done) produce();
  }
  if (!convert_step(0)) {
    give_up();
    return;
  }

  // per-thread state
  const unsigned span = (unsigned)(P.ns - 2 * P.tau - 2);   // valid iff 0 <= it - tau <= span
  const float2 kTwo23x2 = make_float2(8388608.0f, 8388608.0f);
  const float2 kMinusTwo23x2 = make_float2(-8388608.0f, -8388608.0f);
  const float2 kMinusOne2 = make_float2(-1.0f, -1.0f);
  float Tsmp = 0.f, T2smp = 0.f;
  constexpr int RP = (RC + 1) / 2;
  float2 ca2[RP], cb2[RP], cc2[RP];
  auto CA = [&](int r) { return (r & 1) ? ca2[r >> 1].y : ca2[r >> 1].x; };
  auto CB = [&](int r) { return (r & 1) ? cb2[r >> 1].y : cb2[r >> 1].x; };
  auto CC = [&](int r) { return (r & 1) ? cc2[r >> 1].y : cc2[r >> 1].x; };
  AccSet<W, LAY, RC> fa;
  int ntask = 0;
  float last_s = 0.f;
  int last_i = 0x7fffffff;

  for (int c = 0;; ++c) {
    const ChunkTag tg = *tag_at(c);   // visible: this thread saw chunk c's raw barrier complete
    if (tg.flags & CH_END) break;
    // convert the next chunk (it exists: this one is not the end)
    if (!convert_step(c + 1)) {
      give_up();
      return;
    }
    // every warp has converted chunk c
    if (!wait_bar(&q_full[c % kStages], (c / kStages) & 1)) {
      give_up();
      return;
    }
    // the raw buffer of chunk c is free: warp (c+2) % nwarps plans chunk c+2 into
    // it.  That warp has seen chunk c+1's copies armed, i.e. its planning done.
    if (warp == (c + 2) % nwarps && !prod->done) produce();

    const ChunkMeta* meta = meta_at(c);
    if (tg.flags & CH_PASS_FIRST) {
      if (tg.pass == 0) {
        const int t0 = min(tg.t0s + lane, P.ns - 1);
        Tsmp = (float)t0;
        T2smp = Tsmp * Tsmp;
      }
      const float4* cand = P.cand + tg.pass * P.cpp + warp * RC;
#pragma unroll
      for (int r = 0; r < 2 * RP; ++r) {
        const float4 cv = __ldg(cand + min(r, RC - 1));
        if (r & 1) {
          ca2[r >> 1].y = cv.x;
          cb2[r >> 1].y = cv.y;
          cc2[r >> 1].y = cv.z;
        } else {
          ca2[r >> 1].x = cv.x;
          cb2[r >> 1].x = cv.y;
          cc2[r >> 1].x = cv.z;
        }
      }
#pragma unroll
      for (int r = 0; r < RC; ++r) {
        fa[r].reset();
        kahan_hi[r * NT + threadIdx.x] = 0.f;
        kahan_lo[r * NT + threadIdx.x] = 0.f;
      }
    }

    // ---- compute chunk c ----
    {
      const int n = meta->n, n_in = meta->n_in;
      const uint32_t bufq_addr = smem_u32(quad_at(c));
      const uint32_t top = bufq_addr + EB * (uint32_t)P.cap;
      // LAY_FT: side entry address of main entry address a is a / 2 + side_shift
      const uint32_t side_shift = bufq_addr + 16u * (uint32_t)(P.cap + kZeroSlots) - (bufq_addr >> 1);
      const float2 Tsmp2 = make_float2(Tsmp, Tsmp);
      const float2 T2smp2 = make_float2(T2smp, T2smp);
      // traces on which every item is in range: traveltimes of item pairs in
      // FP32x2, address = bits(t + 2^23) * EB + base (mod 2^32), clamped to the
      // stage as a guard
#pragma unroll TU
      for (int e = 0; e < n_in; ++e) {
        const float4 g = meta->geo[e];
        const uint32_t base = bufq_addr + EB * (uint32_t)(__float_as_int(g.w) - P.tau) - EB * 0x4B000000u;
        const float2 gx2 = make_float2(g.x, g.x), gy2 = make_float2(g.y, g.y), gz2 = make_float2(g.z, g.z);
        float2 q02 = make_float2(0.f, 0.f);
        if (BRUN && METHOD == METHOD_CRS) {
          // B-run candidates share A and C: (t0 + A|dm|)^2 + C h once per trace
          const float u0 = fmaf(CA(0), g.x, Tsmp);
          const float q0 = fmaf(u0, u0, CC(0) * g.z);
          q02 = make_float2(q0, q0);
        }
#pragma unroll
        for (int rp = 0; rp < RP; ++rp) {
          float2 t2;
          if (METHOD == METHOD_CMP) {
            t2 = __ffma2_rn(cc2[rp], gz2, T2smp2);
          } else if (BRUN) {
            t2 = __ffma2_rn(cb2[rp], gy2, q02);
          } else {
            const float2 u = __ffma2_rn(ca2[rp], gx2, Tsmp2);
            t2 = __ffma2_rn(u, u, __ffma2_rn(cb2[rp], gy2, __fmul2_rn(cc2[rp], gz2)));
          }
          const float2 t = make_float2(sqrt_fast(t2.x), sqrt_fast(t2.y));
          const float2 y = __fadd2_rz(t, kTwo23x2);
          const float2 x = __ffma2_rn(__fadd2_rn(y, kMinusTwo23x2), kMinusOne2, t);   // t - floor(t)
          if constexpr (SEMB_CHECKED) {
            const int i0 = __float_as_int(g.w) - P.tau - 0x4B000000;
            const int t0c = min(tg.t0s + lane, P.ns - 1);
            report_window(P.status, __float_as_int(y.x) + i0, W, src_at(c)[e], tg.cdp, t0c);
            if (2 * rp + 1 < RC) report_window(P.status, __float_as_int(y.y) + i0, W, src_at(c)[e], tg.cdp, t0c);
          }
          if constexpr (LAY == LAY_FT) {
            // main entry a (16 bytes per sample), side entry a / 2 + side_shift (8 bytes)
            const uint32_t a0 = min(__float_as_uint(y.x) * EB + base, top);
            fa[2 * rp].add_ft(a0, (a0 >> 1) + side_shift, t.x);
            if (2 * rp + 1 < RC) {
              const uint32_t a1 = min(__float_as_uint(y.y) * EB + base, top);
              fa[2 * rp + 1].add_ft(a1, (a1 >> 1) + side_shift, t.y);
            }
          } else if constexpr (LAY == LAY_X3) {
            // both items of the pair in one set of FP32x2 operations
            const uint32_t a0 = min(__float_as_uint(y.x) * EB + base, top);
            if (2 * rp + 1 < RC) {
              fa.add_pair(rp, a0, min(__float_as_uint(y.y) * EB + base, top), x);
            } else {
              fa[2 * rp].add(a0, x.x);
            }
          } else {
            fa[2 * rp].add(min(__float_as_uint(y.x) * EB + base, top), x.x);
            if (2 * rp + 1 < RC) fa[2 * rp + 1].add(min(__float_as_uint(y.y) * EB + base, top), x.y);
          }
        }
      }
      // the other traces: per-item range checks; an out-of-range item reads the
      // zero block with weight 0 and does not count
      for (int e = kMaxChunk - (n - n_in); e < kMaxChunk; ++e) {
        const float4 g = meta->geo[e];
        const int soff = __float_as_int(g.w);
        float q0 = 0.f;
        if (BRUN && METHOD == METHOD_CRS) {
          const float u0 = fmaf(CA(0), g.x, Tsmp);
          q0 = fmaf(u0, u0, CC(0) * g.z);
        }
        if (GLOB && soff == kGlobalEntry) {
          // a window larger than a stage: the items read the FP32 store
          if constexpr (GLOB) global_entry<METHOD, BRUN>(P, meta->raw[e], g, q0, Tsmp, T2smp, span, ca2, cb2, cc2, fa.a);
          continue;
        }
#pragma unroll
        for (int r = 0; r < RC; ++r) {
          float t2;
          if (METHOD == METHOD_CMP) {
            t2 = fmaf(CC(r), g.z, T2smp);
          } else if (BRUN) {
            t2 = fmaf(CB(r), g.y, q0);
          } else {
            const float u = fmaf(CA(r), g.x, Tsmp);
            t2 = fmaf(u, u, fmaf(CB(r), g.y, CC(r) * g.z));
          }
          const float t = sqrt_fast(t2);   // NaN for t2 < 0: out of range below
          const float y = __fadd_rz(t, 8388608.0f);
          const int rel = __float_as_int(y) - (0x4B000000 + P.tau);   // it - tau
          const bool ok = (unsigned)rel <= span;
          const float x = ok ? t - (y - 8388608.0f) : 0.0f;
          const unsigned idx = min(ok ? (unsigned)(soff + rel) : (unsigned)P.cap, (unsigned)P.cap);
          if constexpr (SEMB_CHECKED) {
            if (ok) report_window(P.status, soff + rel, W, src_at(c)[e], tg.cdp, min(tg.t0s + lane, P.ns - 1));
          }
          if constexpr (LAY == LAY_FT) {
            const uint32_t a = bufq_addr + EB * idx;
            fa[r].add_ft(a, (a >> 1) + side_shift, ok ? t : 0.0f);
          } else {
            fa[r].add(bufq_addr + EB * idx, x);
          }
          fa[r].M += ok ? 1 : 0;
        }
      }
#pragma unroll
      for (int r = 0; r < RC; ++r) {
        fa[r].M += n_in;   // in-range traces count for every item
        // Kahan: fold this chunk's energy into the compensated total
        const int o = r * NT + threadIdx.x;
        const float hi = kahan_hi[o], lo = kahan_lo[o];
        const float yv = fa[r].take_energy() - lo;
        const float tv = hi + yv;
        kahan_lo[o] = (tv - hi) - yv;
        kahan_hi[o] = tv;
      }
    }
    // quad stage and metadata of chunk c are no longer read by this warp
    __syncwarp();
    if (lane == 0) mbar_arrive(&q_empty[c % kStages]);

    if (!(tg.flags & CH_PASS_LAST)) continue;

    // ---- finalize the pass's items into this thread's top-4 ----
    if (tg.pass == 0) {
      // the first pass of a task: the previous task's merge must have read the lists
      if (ntask > 0 && !wait_bar(merge_done, (ntask - 1) & 1)) {
        give_up();
        return;
      }
#pragma unroll
      for (int q = 0; q < K; ++q) {
        top_s[q * NT + threadIdx.x] = 0.f;
        top_i[q * NT + threadIdx.x] = 0x7fffffff;
        top_k[q * NT + threadIdx.x] = 0.f;
      }
      last_s = 0.f;
      last_i = 0x7fffffff;
    }
    const float4* cand = P.cand + tg.pass * P.cpp + warp * RC;
#pragma unroll
    for (int r = 0; r < RC; ++r) {
      float zden = 0.f;
      if constexpr (Z0) {
        // the central traces' sums of this item's C index
        const int gi = __float_as_int(__ldg(&cand[r].w));
        if (gi >= 0) {
          const float* z = z0_slot(tg.zslot) + (gi % P.nc_grid - tg.ic_lo) * 5 * 32 + lane;
          fa[r].add_sums(z[0], z[32], z[64]);
          zden = z[96];
          fa[r].M += (int)z[128];
        }
      }
      float acsq, lin;
      fa[r].sums(acsq, lin);
      const float den = kahan_hi[r * NT + threadIdx.x] - kahan_lo[r * NT + threadIdx.x] + zden;
      const float mf = (float)fa[r].M;
      const int err = tg.napert - fa[r].M;
      const bool ok = (den > kEpsilonF) && (fa[r].M > 0) && (err < 2);
      const float sem = ok ? __fdividef(acsq, den * mf) : kSent;
      const float stk = ok ? __fdividef(lin, (float)W * mf) : kSent;
      const int idx = __float_as_int(__ldg(&cand[r].w));   // -1: padding slot
      if (idx >= 0 && sem > 0.f && better(sem, idx, last_s, last_i)) {
        // sorted insert (descending semblance, ascending index)
        float cs = sem, ck = stk;
        int cidx = idx;
#pragma unroll
        for (int q = 0; q < K; ++q) {
          const int o = q * NT + threadIdx.x;
          const float bs = top_s[o];
          const int bi = top_i[o];
          if (better(cs, cidx, bs, bi)) {
            const float bk = top_k[o];
            top_s[o] = cs;
            top_i[o] = cidx;
            top_k[o] = ck;
            cs = bs;
            cidx = bi;
            ck = bk;
          }
        }
        last_s = top_s[(K - 1) * NT + threadIdx.x];
        last_i = top_i[(K - 1) * NT + threadIdx.x];
      }
    }
    if (!(tg.flags & CH_TASK_LAST)) continue;

    // ---- task done for this warp; the last warp to get here merges ----
    __threadfence_block();
    __syncwarp();
    int last = 0;
    if (lane == 0) last = atomicAdd(merge_cnt, 1) == nwarps - 1;
    last = __shfl_sync(0xffffffffu, last, 0);
    if (last) {
      __threadfence_block();
      float fs[K], fk[K];
      int fi[K];
#pragma unroll
      for (int q = 0; q < K; ++q) {
        fs[q] = 0.f;
        fi[q] = 0x7fffffff;
        fk[q] = 0.f;
      }
      for (int w2 = 0; w2 < nwarps; ++w2) {
        for (int q2 = 0; q2 < K; ++q2) {
          float cs = top_s[q2 * NT + w2 * 32 + lane];
          int cidx = top_i[q2 * NT + w2 * 32 + lane];
          float ck = top_k[q2 * NT + w2 * 32 + lane];
          if (!(cs > 0.f)) continue;
#pragma unroll
          for (int q = 0; q < K; ++q) {
            if (better(cs, cidx, fs[q], fi[q])) {
              const float ts = fs[q], tk = fk[q];
              const int ti = fi[q];
              fs[q] = cs;
              fi[q] = cidx;
              fk[q] = ck;
              cs = ts;
              cidx = ti;
              ck = tk;
            }
          }
        }
      }
      const int tt = tg.t0s + lane;
      if (tt < P.ns) {
        const int64_t o = (int64_t)tg.cdp * P.ns + tt;
#pragma unroll
        for (int q = 0; q < K; ++q) {
          P.top_sem[o * kTopK + q] = fs[q];
          P.top_idx[o * kTopK + q] = fs[q] > 0.f ? fi[q] : -1;
          P.top_stk[o * kTopK + q] = fk[q];
        }
      }
      __syncwarp();
      if (lane == 0) {
        *merge_cnt = 0;
        mbar_arrive(merge_done);   // the lists may be reused
      }
    }
    ++ntask;
  }
}

}  // namespace semb
