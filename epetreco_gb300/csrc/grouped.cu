// grouped.cu -- a reconstruction's system matrix as row groups with
// group-local column ids, and the one-pass MLEM iteration over it.
//
// The rows (in the reconstruction's crystal-pair order) are cut into groups
// of consecutive rows whose distinct columns fit a per-warp table in shared
// memory.  Consecutive rows in that order are a fan of lines through nearly
// one point, so a group touches few voxels: at 52^3 voxels a group of 32
// rows (~14k entries) touches ~1000.  Each entry keeps only its value and a
// 2-byte rank of its column among the group's sorted distinct columns (the
// group's table), 6 bytes per entry in FP32 and 4 in BF16/FP16 instead of a
// CSR plus a column-major copy (16 bytes).  Rows start on 4-entry boundaries
// and are padded to whole 4-entry chunks with zero values whose rank is a
// trash slot (past the table), so the pass reads 16-byte chunks with no
// per-entry bounds tests.
//
// One iteration reads every entry once (k_group_mlem): a warp takes a group,
// gathers x at the table into shared memory, and row by row forms A x from
// the shared copy, e = y / (A x) and adds the row times e into the group's
// shared correction; a row's columns are distinct, so the lanes never write
// the same word (padding goes to the trash slot, which is never read) and
// each column's sum runs in row order.  The group's corrections go to one
// slot per (group, column); the slots of each column, listed in group order
// (built once: the column-major order of the table's entries), are summed in
// that order by the slot-sum kernel (k_sums), whose epilogue applies x*c/s.
// Every sum has an input-determined order, so results are deterministic.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "internal.h"
#include "mlem_internal.h"
#include "spmv.cuh"

namespace epet {

constexpr int kGroupFirstRows = 32;  // rows of a first-cut group (split while too wide)
constexpr int kGroupThreads = 256;   // threads of the table-building kernels
constexpr int kTrash = kGroupCap;    // rank of the padding entries
// Shared tables are indexed by rank (the word of rank r sits in bank r % 32).
// A row's entries are stored so that each warp-wide shared access of the
// pass takes 32 consecutive entries of the row (k_group_tables): their ranks
// ascend by a few, which spreads them over the banks better than the fixed
// swizzles of the ranks tried: 2.05 distinct-address wavefronts per 32
// entries on rows of the full workload, against 2.94 with a lane taking 4
// consecutive entries and the ranks swizzled as r + r / 32 (the pass 7 %
// faster).  A layout balancing each row over the banks (1.27 wavefronts)
// was no faster: the pass is bound by the latency of its entry stream.
__host__ __device__ constexpr int sw_rank(int r) { return r; }
constexpr int kGroupStride = sw_rank(kGroupCap) + 4;  // floats per shared table (trash included)
constexpr size_t kGroupSmem = (size_t)kGroupWarps * 2 * kGroupStride * 4;
static_assert(kGroupSmem <= 227 * 1024, "grouped tables exceed shared memory");

// Row r of the source: its columns and values, and its length.
struct RowSpan {
  const int32_t* col;
  const float* val;
  int64_t n;
};
__device__ __forceinline__ RowSpan row_span(const RowSource& A, int64_t r) {
  if (A.segs) {
    const int64_t q = A.idx[r];
    const SegDev sg = A.segs[q / A.ch];
    const int64_t b = A.rp[q] - sg.e0;
    return RowSpan{sg.col + b, sg.val + b, A.rp[q + 1] - A.rp[q]};
  }
  const int64_t b = A.rp[r];
  return RowSpan{A.col + b, A.val + b, A.rp[r + 1] - b};
}

// The spans of rows r0 .. r1 - 1 (at most kGroupFirstRows) in shared memory,
// with their exclusive prefix off[] (off[nr] = the group's entries); the
// loads run in parallel, a thread per row.  Ends with a block barrier.
struct GroupSpans {
  const int32_t* col[kGroupFirstRows];
  const float* val[kGroupFirstRows];
  int off[kGroupFirstRows + 1];
};
__device__ __forceinline__ void load_spans(const RowSource& A, int r0, int r1, GroupSpans* S) {
  const int nr = r1 - r0;
  int n = 0;
  if ((int)threadIdx.x < nr) {
    const RowSpan rs = row_span(A, r0 + threadIdx.x);
    S->col[threadIdx.x] = rs.col;
    S->val[threadIdx.x] = rs.val;
    n = (int)rs.n;
  }
  if (threadIdx.x < 32) {  // nr <= 32: one warp's scan
    const int inc = warp_incl_scan(n);
    if ((int)threadIdx.x < nr) S->off[threadIdx.x + 1] = inc;
    if (threadIdx.x == 0) S->off[0] = 0;
  }
  __syncthreads();
}

// Sets the group's columns in the bitmap bm: a warp per row, its lanes
// along the row, four column loads issued before their atomics.
__device__ __forceinline__ void set_group_columns(const GroupSpans& S, int nr, unsigned* bm) {
  const int lane = threadIdx.x & 31;
  for (int r = threadIdx.x >> 5; r < nr; r += kGroupThreads / 32) {
    const int32_t* col = S.col[r];
    const int n = S.off[r + 1] - S.off[r];
    for (int j0 = lane; j0 < n; j0 += 128) {
      int v[4];
#pragma unroll
      for (int u = 0; u < 4; u++) v[u] = j0 + 32 * u < n ? col[j0 + 32 * u] : -1;
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (v[u] >= 0) atomicOr(&bm[v[u] >> 5], 1u << (v[u] & 31));
    }
  }
}

// Distinct columns of the candidate groups cand[g] = {r0, r1}: a bitmap over
// the columns in shared memory (nwords 32-bit words).
__global__ void __launch_bounds__(kGroupThreads)
k_group_distinct(RowSource A, const int2* __restrict__ cand, int nwords,
                 int32_t* __restrict__ nd) {
  extern __shared__ unsigned gbm[];
  __shared__ int wsum[kGroupThreads / 32];
  __shared__ GroupSpans S;
  for (int i = threadIdx.x; i < nwords; i += kGroupThreads) gbm[i] = 0u;
  const int2 c = cand[blockIdx.x];
  load_spans(A, c.x, c.y, &S);
  set_group_columns(S, c.y - c.x, gbm);
  __syncthreads();
  int n = 0;
  for (int i = threadIdx.x; i < nwords; i += kGroupThreads) n += __popc(gbm[i]);
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < kGroupThreads / 32; w++) t += wsum[w];
    nd[blockIdx.x] = t;
  }
}

// Storage order of a row of nq 4-entry chunks (its entries j in CSR order,
// then padding): the pass hands chunk 32 u + l to lane l in round u and
// reads position t of every lane's chunk with one shared access, so the
// entries are placed for this access to take consecutive entries: round u
// (cq = min(32, nq - 32 u) chunks) holds entry j = 128 u + t cq + l at chunk
// l, position t, i.e. at 128 u + 4 l + t.

// Tables and the padded layout of the final groups (one block per group):
// the group's distinct columns, ascending, at table[tb ..]; every row r's
// entries at ptr[r] (a multiple of 4) onwards in the storage order above,
// each as its value and its column's rank among the group's columns, then
// zero values on the trash rank up to the next multiple of 4.  A single row
// wider than the shared tables (a "wide" group) keeps its own columns as its
// table (padded like the row with column 0) and the CSR order; its padding
// points past the row in that table.
//
// Two launches.  The first (nd_out set, groups null, table the scratch
// ftab) takes the first cuts, block b the rows [32 b, min(m, 32 b + 32)): it
// writes each cut's count of distinct columns to nd_out[b] and, for a cut
// that fits the shared tables, its table at ftab + b * kGroupCap and its
// entries.  The second takes the final groups: a first cut kept whole
// copies its table from ftab to its slots; the groups made by splitting
// wider cuts are laid out in full.
__global__ void __launch_bounds__(kGroupThreads, 8)
k_group_tables(RowSource A, const GroupDesc* __restrict__ groups, int64_t m, int nwords,
               const int64_t* __restrict__ ptr, int32_t* __restrict__ table,
               const int32_t* __restrict__ ftab, int32_t* __restrict__ nd_out,
               float* __restrict__ pval, uint16_t* __restrict__ ploc) {
  extern __shared__ unsigned gsh[];
  unsigned* bm = gsh;
  // per bitmap word the rank of its first column (< kGroupCap where read):
  // 16 bits keep the block at 6 bytes per word (8 blocks per SM at 52^3)
  uint16_t* pre = reinterpret_cast<uint16_t*>(gsh + nwords);
  __shared__ int wtot[kGroupThreads / 32];
  __shared__ int s_nd;
  const bool first = nd_out != nullptr;
  GroupDesc gd;
  if (first) {
    const int64_t r0 = (int64_t)blockIdx.x * kGroupFirstRows;
    gd = GroupDesc{(int32_t)r0, (int32_t)min(m, r0 + kGroupFirstRows), 0, 0};
  } else {
    gd = groups[blockIdx.x];
    if (gd.nd <= kGroupCap && gd.r0 % kGroupFirstRows == 0 &&
        gd.r1 == min(m, (int64_t)gd.r0 + kGroupFirstRows)) {
      // a first cut kept whole: laid out by the first launch
      const int32_t* src = ftab + (int64_t)(gd.r0 / kGroupFirstRows) * kGroupCap;
      for (int j = threadIdx.x; j < gd.nd; j += kGroupThreads) table[gd.tb + j] = src[j];
      return;
    }
  }
  if (!first && gd.nd > kGroupCap) {  // wide: one row
    const RowSpan rs = row_span(A, gd.r0);
    const int64_t d = ptr[gd.r0], pn = ptr[gd.r0 + 1] - d;
    for (int64_t j = threadIdx.x; j < gd.nd; j += kGroupThreads)
      table[gd.tb + j] = j < rs.n ? rs.col[j] : 0;
    for (int64_t j = threadIdx.x; j < pn; j += kGroupThreads) {
      pval[d + j] = j < rs.n ? rs.val[j] : 0.f;
      ploc[d + j] = 0;  // (unused: a wide row reads its table by position)
    }
    return;
  }
  __shared__ GroupSpans S;
  const int nr = gd.r1 - gd.r0;
  for (int i = threadIdx.x; i < nwords; i += kGroupThreads) bm[i] = 0u;
  load_spans(A, gd.r0, gd.r1, &S);
  set_group_columns(S, nr, bm);
  __syncthreads();
  // exclusive prefix of the words' popcounts: thread t owns a contiguous
  // range of words
  const int per = (nwords + kGroupThreads - 1) / kGroupThreads;
  const int wb = min(nwords, (int)threadIdx.x * per), we = min(nwords, wb + per);
  int cnt = 0;
  for (int w = wb; w < we; w++) cnt += __popc(bm[w]);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int inc = warp_incl_scan(cnt);
  if (lane == 31) wtot[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    const int t = lane < kGroupThreads / 32 ? wtot[lane] : 0;
    const int ti = warp_incl_scan(t);
    if (lane < kGroupThreads / 32) wtot[lane] = ti - t;
    if (lane == kGroupThreads / 32 - 1) s_nd = ti;
  }
  __syncthreads();
  if (first) {  // (uniform across the block)
    if (threadIdx.x == 0) nd_out[blockIdx.x] = s_nd;
    if (s_nd > kGroupCap) return;  // split by the host, laid out by the second launch
  }
  // (the first launch's table is its cut's share of the scratch ftab)
  int32_t* const tab = first ? table + (int64_t)blockIdx.x * kGroupCap : table + gd.tb;
  int run = wtot[wid] + inc - cnt;
  for (int w = wb; w < we; w++) {
    pre[w] = (uint16_t)run;
    unsigned word = bm[w];
    while (word) {
      const int bit = __ffs(word) - 1;
      tab[run] = w * 32 + bit;
      run++;
      word &= word - 1u;
    }
  }
  __syncthreads();
  // the padded layout a 4-entry chunk at a time, a warp per row: lane l
  // takes chunk l of every round u, which holds the row's entries j = 128 u
  // + t cq + l (t = 0..3, the storage order above), padding (j past the row)
  // as zero values on the trash rank; a chunk's values and ranks are
  // written with one 16-byte and one 8-byte store
  for (int r = wid; r < nr; r += kGroupThreads / 32) {
    const int32_t* col = S.col[r];
    const float* val = S.val[r];
    const int n = S.off[r + 1] - S.off[r];
    const int64_t d = ptr[gd.r0 + r];
    const int nq = (int)((ptr[gd.r0 + r + 1] - d) >> 2);
    for (int c = lane; c < nq; c += 32) {
      const int u = c >> 5;
      const int cq = min(32, nq - 32 * u);
      int cc[4];
      float vv[4];
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const int j = 128 * u + t * cq + lane;
        cc[t] = j < n ? col[j] : -1;
        vv[t] = j < n ? val[j] : 0.f;
      }
      unsigned rk[4];
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const unsigned v = (unsigned)cc[t];
        rk[t] = cc[t] >= 0
                    ? (unsigned)sw_rank(pre[v >> 5] + __popc(bm[v >> 5] & ((1u << (v & 31)) - 1u)))
                    : (unsigned)sw_rank(kTrash);
      }
      *reinterpret_cast<float4*>(pval + d + 4 * c) = make_float4(vv[0], vv[1], vv[2], vv[3]);
      *reinterpret_cast<uint2*>(ploc + d + 4 * c) = make_uint2(rk[0] | (rk[1] << 16),
                                                               rk[2] | (rk[3] << 16));
    }
  }
}

// Dynamic shared memory of k_group_tables: the bitmap and the word ranks.
static size_t table_smem(int nwords) { return (size_t)nwords * 6; }

__global__ void k_padded_len(RowSource A, int64_t m, int64_t* __restrict__ len) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m) return;
  const int64_t q = A.segs ? A.idx[r] : r;
  len[r] = (A.rp[q + 1] - A.rp[q] + 3) & ~int64_t(3);
}

__global__ void k_fill_f32(float* __restrict__ p, int64_t n, float v) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

epet_status grouped_ones(GroupedMatrix* G, cudaStream_t st) {
  if (G->ones) return EPET_OK;
  const int64_t ns = std::max<int64_t>(G->nslots, 1);
  EPET_CUDA(dev_alloc((void**)&G->ones, ns * 4, st));
  if (G->nslots > 0) {
    k_fill_f32<<<ceil_div(G->nslots, 256), 256, 0, st>>>(G->ones, G->nslots, 1.f);
    EPET_LAUNCHED();
  }
  return EPET_OK;
}

// 16-bit values: q = the 16-bit float of value / scale, scale = the row's
// largest value (the 16-bit forms' quantisation), a warp per row.
template <int FMT>
__device__ __forceinline__ uint16_t gq_to(float v) {
  if (FMT == 1) return __bfloat16_as_ushort(__float2bfloat16_rn(v));
  return __half_as_ushort(__float2half_rn(v));
}
template <int FMT>
__device__ __forceinline__ float gq_from(uint32_t q) {
  if (FMT == 1) return __uint_as_float(q << 16);
  return __half2float(__ushort_as_half((unsigned short)q));
}

template <int FMT>
__global__ void k_group_quantise(const int64_t* __restrict__ ptr, const float* __restrict__ val,
                                 int64_t m, float* __restrict__ scale, uint16_t* __restrict__ q) {
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= m) return;
  const int64_t b = ptr[r], e = ptr[r + 1];
  float mx = 0.f;
  for (int64_t k = b + lane; k < e; k += 32) mx = fmaxf(mx, fabsf(val[k]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const float sc = mx > 0.f ? mx : 1.f;
  if (lane == 0) scale[r] = sc;
  for (int64_t k = b + lane; k < e; k += 32) q[k] = gq_to<FMT>(__fdiv_rn(val[k], sc));
}

// A row's entries as the pass holds them: 4-entry chunks, chunk u of lane l
// the (l + 32 u)-th chunk of the (padded) row; values raw (FP32: float4,
// 16-bit: 4 x 16 bits) and column ranks as 4 x 16 bits.
constexpr int kGroupRounds = 4;  // chunks per lane held in registers (512 entries a row)
template <int FMT>
struct RowBuf {
  using V = typename std::conditional<FMT == 0, float4, uint2>::type;
  V v[kGroupRounds];
  uint2 l[kGroupRounds];
};

__device__ __forceinline__ float gval4(const float4& c, int t) {
  return t == 0 ? c.x : t == 1 ? c.y : t == 2 ? c.z : c.w;
}
template <int FMT>
__device__ __forceinline__ float gval(const typename RowBuf<FMT>::V& c, int t) {
  if constexpr (FMT == 0) {
    return gval4(c, t);
  } else {
    const uint32_t w = t < 2 ? c.x : c.y;
    return gq_from<FMT>((t & 1) ? (w >> 16) : (w & 0xffffu));
  }
}
__device__ __forceinline__ int grank(const uint2& c, int t) {
  const uint32_t w = t < 2 ? c.x : c.y;
  return (int)((t & 1) ? (w >> 16) : (w & 0xffffu));
}

template <int FMT>
__device__ __forceinline__ void gload_chunk(const void* __restrict__ val,
                                            const uint16_t* __restrict__ loc, int64_t k4,
                                            typename RowBuf<FMT>::V* v, uint2* l) {
  if constexpr (FMT == 0)
    *v = __ldcs(reinterpret_cast<const float4*>(static_cast<const float*>(val) + k4));
  else
    *v = __ldcs(reinterpret_cast<const uint2*>(static_cast<const uint16_t*>(val) + k4));
  *l = __ldcs(reinterpret_cast<const uint2*>(loc + k4));
}

struct GroupIterArgs {
  const GroupDesc* groups;
  int64_t ngroups;
  const int64_t* row_ptr;  // padded (multiples of 4)
  const void* val;         // float (FP32) or 16-bit bits, padded
  const float* scale;      // per row (16-bit forms)
  const uint16_t* loc;     // padded
  const int32_t* table;
  const float* x;
  const float* y;
  float* ybar;
  float* partial;
};

// What a group's pass needs before its first row: its row pointers, counts
// and scales, one row per lane (a group has at most 32 rows), loaded one
// group ahead.
struct GroupHead {
  GroupDesc gd;
  int64_t rp, rp_end;
  float y, sc;
};

template <int FMT>
__device__ __forceinline__ GroupHead group_head(const GroupIterArgs& a, const GroupDesc& gd,
                                                int lane) {
  GroupHead h;
  h.gd = gd;
  const int nr = gd.r1 - gd.r0;
  h.rp = lane <= nr ? a.row_ptr[gd.r0 + lane] : 0;
  h.rp_end = a.row_ptr[gd.r1];
  h.y = lane < nr ? a.y[gd.r0 + lane] : 0.f;
  h.sc = FMT != 0 && lane < nr ? a.scale[gd.r0 + lane] : 1.f;
  return h;
}

// One group of the MLEM pass (a warp): per row ybar = A x, e = y / ybar (0
// where ybar == 0, the fused epilogue's guard) and the row's share of A^T e
// added, row after row, to the group's shared correction, written to
// partial[slot] at the end.  The next row's entries are in flight while a
// row is reduced and scattered.
// Which groups a pass instantiation handles: kOrdinary (tables in shared
// memory), kWide (one row wider than the shared tables, its own columns as
// its table, read from global memory), or kAny (decided per group).  The
// ordinary groups' kernel carries none of the wide path's instructions:
// with them (kAny) the full-size iteration took 4.85 ms instead of 4.16.
enum GroupKind { kOrdinary = 0, kWide = 1, kAny = 2 };

template <int FMT, int KIND>
__device__ __forceinline__ void group_pass_as(const GroupIterArgs& a, const GroupHead& H,
                                              float* xs, float* cs, int lane) {
  const GroupDesc& gd = H.gd;
  const int nr = gd.r1 - gd.r0;  // <= 32
  const bool wide = KIND == kAny ? gd.nd > kGroupCap : KIND == kWide;
  float yb_l = 0.f;
  auto row_begin = [&](int i) -> int64_t { return __shfl_sync(0xffffffffu, H.rp, i); };
  auto row_end = [&](int i) -> int64_t {
    const int64_t t = __shfl_sync(0xffffffffu, H.rp, (i + 1) & 31);
    return i + 1 < 32 ? t : H.rp_end;
  };
  if (!wide) {
    // x at the table: batches of 8 independent table loads, then their x
    // gathers
    for (int j0 = 0; j0 < gd.nd; j0 += 8 * 32) {
      int col[8];
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int j = j0 + 32 * k + lane;
        col[k] = j < gd.nd ? __ldg(a.table + gd.tb + j) : 0;
      }
#pragma unroll
      for (int k = 0; k < 8; k++) {
        const int j = j0 + 32 * k + lane;
        const float xv = __ldg(a.x + col[k]);
        if (j < gd.nd) {
          xs[sw_rank(j)] = xv;
          cs[sw_rank(j)] = 0.f;
        }
      }
    }
    if (lane == 0) xs[sw_rank(kTrash)] = 0.f;
    __syncwarp();
  }
  auto load_row = [&](int i, RowBuf<FMT>& B) {
    const int64_t b = row_begin(i);
    const int nq = (int)((row_end(i) - b) >> 2);
#pragma unroll
    for (int u = 0; u < kGroupRounds; u++) {
      const int q = lane + 32 * u;
      if (q < nq) gload_chunk<FMT>(a.val, a.loc, b + 4 * q, &B.v[u], &B.l[u]);
    }
  };
  auto process_row = [&](int i, const RowBuf<FMT>& B) {
    const int64_t b = row_begin(i);
    const int nq = (int)((row_end(i) - b) >> 2);
    // dot product: four accumulators (entry position t in its chunk), the
    // shared x loads independent; padding entries are zero
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    auto dot = [&](const typename RowBuf<FMT>::V& vv, const uint2& ll, int q) {
      float xv[4];
#pragma unroll
      for (int t = 0; t < 4; t++)
        xv[t] = wide ? __ldg(a.x + a.table[gd.tb + 4 * q + t]) : xs[grank(ll, t)];
#pragma unroll
      for (int t = 0; t < 4; t++) acc[t] = fmaf(gval<FMT>(vv, t), xv[t], acc[t]);
    };
#pragma unroll
    for (int u = 0; u < kGroupRounds; u++) {
      const int q = lane + 32 * u;
      if (q < nq) dot(B.v[u], B.l[u], q);
    }
    for (int q = lane + 32 * kGroupRounds; q < nq; q += 32) {  // rows over 512 entries
      typename RowBuf<FMT>::V vv;
      uint2 ll;
      gload_chunk<FMT>(a.val, a.loc, b + 4 * q, &vv, &ll);
      dot(vv, ll, q);
    }
    float d = fadd(fadd(acc[0], acc[1]), fadd(acc[2], acc[3]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    const float sc = __shfl_sync(0xffffffffu, H.sc, i);
    const float yb = FMT == 0 ? d : fmul(d, sc);
    if (lane == i) yb_l = yb;
    // e = y / (A x) (mlemOperations.hpp:22-32; 0 where A x == 0)
    const float yr = __shfl_sync(0xffffffffu, H.y, i);
    const float er = yb > 0.f ? __fdiv_rn(yr, yb) : 0.f;
    const float f = FMT == 0 ? er : fmul(er, sc);
    // scatter into the group's correction, a chunk at a time: its four
    // columns are distinct (as all of a row's; padding goes to the trash
    // slot), so the four sums are read before any is written
    auto scatter = [&](const typename RowBuf<FMT>::V& vv, const uint2& ll, int q) {
      if (wide) {
#pragma unroll
        for (int t = 0; t < 4; t++) a.partial[gd.tb + 4 * q + t] = fmul(gval<FMT>(vv, t), f);
        return;
      }
      float old[4];
#pragma unroll
      for (int t = 0; t < 4; t++) old[t] = cs[grank(ll, t)];
#pragma unroll
      for (int t = 0; t < 4; t++) cs[grank(ll, t)] = fmaf(gval<FMT>(vv, t), f, old[t]);
    };
#pragma unroll
    for (int u = 0; u < kGroupRounds; u++) {
      const int q = lane + 32 * u;
      if (q < nq) scatter(B.v[u], B.l[u], q);
    }
    for (int q = lane + 32 * kGroupRounds; q < nq; q += 32) {
      typename RowBuf<FMT>::V vv;
      uint2 ll;
      gload_chunk<FMT>(a.val, a.loc, b + 4 * q, &vv, &ll);
      scatter(vv, ll, q);
    }
    __syncwarp();
  };
  RowBuf<FMT> b0, b1;
  if (nr > 0) load_row(0, b0);
  for (int i = 0; i < nr; i += 2) {
    if (i + 1 < nr) load_row(i + 1, b1);
    process_row(i, b0);
    if (i + 1 < nr) {
      if (i + 2 < nr) load_row(i + 2, b0);
      process_row(i + 1, b1);
    }
  }
  if (lane < nr) a.ybar[gd.r0 + lane] = yb_l;
  if (!wide) {
    for (int j = lane; j < gd.nd; j += 32) a.partial[gd.tb + j] = cs[sw_rank(j)];
    __syncwarp();
  }
}



// A warp per group, a persistent grid striding over the groups; each warp
// holds its group's tables (x and the correction at the distinct columns)
// in its share of the block's shared memory.  The next group's head is
// loaded one group ahead, descriptors two ahead.
template <int FMT>
__global__ void __launch_bounds__(kGroupWarps * 32, 1)
k_group_mlem(GroupIterArgs a) {
  extern __shared__ __align__(16) float gsm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* xs = gsm + (size_t)w * 2 * kGroupStride;
  float* cs = xs + kGroupStride;
  const int64_t step = (int64_t)gridDim.x * kGroupWarps;
  int64_t g = (int64_t)blockIdx.x * kGroupWarps + w;
  if (g >= a.ngroups) return;
  GroupHead cur = group_head<FMT>(a, a.groups[g], lane);
  GroupDesc nxt = g + step < a.ngroups ? a.groups[g + step] : GroupDesc{0, 0, 0, 0};
  for (; g < a.ngroups; g += step) {
    const GroupDesc nn =
        g + 2 * step < a.ngroups ? a.groups[g + 2 * step] : GroupDesc{0, 0, 0, 0};
    GroupHead head_next{};
    if (g + step < a.ngroups) head_next = group_head<FMT>(a, nxt, lane);
    // (wide groups: k_group_mlem_wide)
    if (cur.gd.nd <= kGroupCap) group_pass_as<FMT, kOrdinary>(a, cur, xs, cs, lane);
    cur = head_next;
    nxt = nn;
  }
}

// The wide groups (ids in wide[0 .. nwide)), a warp each.
template <int FMT>
__global__ void __launch_bounds__(128)
k_group_mlem_wide(GroupIterArgs a, const int32_t* __restrict__ wide, int64_t nwide) {
  const int lane = threadIdx.x & 31;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= nwide) return;
  const GroupHead h = group_head<FMT>(a, a.groups[wide[i]], lane);
  group_pass_as<FMT, kWide>(a, h, nullptr, nullptr, lane);
}

// The same over the groups of many reconstructions (batched form): global
// group g belongs to problem p with gstart[p] <= g < gstart[p + 1].
__global__ void __launch_bounds__(kGroupWarps * 32, 1)
k_group_mlem_batch(const GroupIterArgs* __restrict__ desc, const int64_t* __restrict__ gstart,
                   int np) {
  extern __shared__ __align__(16) float gsm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* xs = gsm + (size_t)w * 2 * kGroupStride;
  float* cs = xs + kGroupStride;
  const int64_t total = gstart[np];
  const int64_t step = (int64_t)gridDim.x * kGroupWarps;
  auto locate = [&](int64_t g) {  // gstart[lo] <= g < gstart[lo + 1]
    int lo = 0, hi = np;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(gstart + mid) <= g) lo = mid;
      else hi = mid;
    }
    return lo;
  };
  int64_t g = (int64_t)blockIdx.x * kGroupWarps + w;
  if (g >= total) return;
  // the problem's descriptor held by value; the next group's problem and
  // head loaded one group ahead
  int p = locate(g);
  GroupIterArgs a = desc[p];
  GroupHead cur = group_head<0>(a, a.groups[g - gstart[p]], lane);
  for (; g < total; g += step) {
    int pn = p;
    GroupHead hn{};
    if (g + step < total) {
      pn = locate(g + step);
      const GroupIterArgs& an = desc[pn];
      hn = group_head<0>(an, an.groups[g + step - gstart[pn]], lane);
    }
    // (wide groups: k_group_mlem_batch_wide)
    if (cur.gd.nd <= kGroupCap) group_pass_as<0, kOrdinary>(a, cur, xs, cs, lane);
    if (pn != p) {
      p = pn;
      a = desc[p];
    }
    cur = hn;
  }
}

// The wide groups of a batch (global group ids wide[0 .. nwide)), a warp each.
__global__ void __launch_bounds__(128)
k_group_mlem_batch_wide(const GroupIterArgs* __restrict__ desc, const int64_t* __restrict__ gstart,
                        int np, const int32_t* __restrict__ wide, int64_t nwide) {
  const int lane = threadIdx.x & 31;
  const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (i >= nwide) return;
  const int64_t g = wide[i];
  int lo = 0, hi = np;  // gstart[lo] <= g < gstart[lo + 1]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(gstart + mid) <= g) lo = mid;
    else hi = mid;
  }
  const GroupIterArgs a = desc[lo];
  const GroupHead h = group_head<0>(a, a.groups[g - gstart[lo]], lane);
  group_pass_as<0, kWide>(a, h, nullptr, nullptr, lane);
}

// Column sums of the grouped matrix's values (the 16-bit forms dequantised)
// over its rows, by the same group / slot structure as the pass: a warp per
// group adds its rows' values, row after row, into the group's shared sums
// (the slots); the slot sums per column then run on the slot-sum kernel.
template <int FMT>
__global__ void __launch_bounds__(kGroupWarps * 32, 1)
k_group_colsum(GroupIterArgs a) {
  extern __shared__ __align__(16) float gsm[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* cs = gsm + (size_t)w * 2 * kGroupStride;
  for (int64_t g = (int64_t)blockIdx.x * kGroupWarps + w; g < a.ngroups;
       g += (int64_t)gridDim.x * kGroupWarps) {
    const GroupDesc gd = a.groups[g];
    const bool wide = gd.nd > kGroupCap;
    if (!wide) {
      for (int j = lane; j < gd.nd; j += 32) cs[sw_rank(j)] = 0.f;
      __syncwarp();
    }
    for (int r = gd.r0; r < gd.r1; r++) {
      const int64_t b = a.row_ptr[r], e = a.row_ptr[r + 1];
      const float sc = FMT == 0 ? 1.f : a.scale[r];
      for (int64_t k = b + lane; k < e; k += 32) {
        float v;
        if constexpr (FMT == 0) v = static_cast<const float*>(a.val)[k];
        else v = fmul(gq_from<FMT>(static_cast<const uint16_t*>(a.val)[k]), sc);
        if (wide) a.partial[gd.tb + (k - b)] = v;
        else cs[a.loc[k]] = fadd(cs[a.loc[k]], v);  // padding: the trash slot
      }
      __syncwarp();
    }
    if (!wide) {
      for (int j = lane; j < gd.nd; j += 32) a.partial[gd.tb + j] = cs[sw_rank(j)];
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------- host

static int bitmap_words(int64_t V) { return (int)((V + 31) / 32); }

bool grouped_supported(int64_t V, int64_t m) {
  // two V-bit maps in a table block's shared memory; int32 rows
  return V > 0 && (size_t)bitmap_words(V) * 8 <= (size_t)200 * 1024 && m < INT32_MAX;
}

void grouped_free(GroupedMatrix* G, cudaStream_t st) {
  for (void* p : {(void*)G->groups, (void*)G->table, (void*)G->loc, (void*)G->wide,
                  (void*)G->cg_ptr,
                  (void*)G->cg_slot, (void*)G->ones, (void*)G->partial, (void*)G->val16,
                  (void*)G->val32, (void*)G->row_ptr, (void*)G->scale})
    if (p) dev_free(p, st);
  *G = GroupedMatrix{};
}

void grouped_drop_fp32(GroupedMatrix* G, cudaStream_t st) {
  if (G->fmt != EPET_VALUES_FP32 && G->val32) {
    dev_free(G->val32, st);
    G->val32 = nullptr;
  }
}

// Where the first round of form_groups lays out the first cuts that fit
// (k_group_tables' first launch): the padded row pointers, the scratch
// tables (kGroupCap per first cut) and the padded values and ranks.
struct FirstCuts {
  const int64_t* ptr;
  int32_t* ftab;
  float* pval;
  uint16_t* ploc;
};

// Groups of consecutive rows of A (row pointers on the device) whose
// distinct columns fit kGroupCap: first cuts of kGroupFirstRows rows, halved
// while too wide; a single row wider than that is a group of its own, its
// table the row's columns padded to whole 4-entry chunks.  The first round
// measures the first cuts and lays out those that fit (FirstCuts); the
// halves are measured by k_group_distinct.
static epet_status form_groups(const RowSource& A, int64_t m, int64_t ncols, const FirstCuts& fc,
                               std::vector<GroupDesc>* out, cudaStream_t st) {
  const int nwords = bitmap_words(ncols);
  const int64_t ncut = (m + kGroupFirstRows - 1) / kGroupFirstRows;
  EPET_CUDA(cudaFuncSetAttribute(k_group_distinct, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 nwords * 4));
  // every first cut counted, those that fit laid out
  std::vector<int32_t> cut_nd(ncut);
  {
    int32_t* nd = nullptr;
    cudaError_t e = dev_alloc((void**)&nd, std::max<int64_t>(ncut, 1) * 4, st);
    if (e == cudaSuccess && ncut > 0) {
      k_group_tables<<<(unsigned)ncut, kGroupThreads, table_smem(nwords), st>>>(
          A, nullptr, m, nwords, fc.ptr, fc.ftab, nullptr, nd, fc.pval, fc.ploc);
      note_launch();
      e = cudaGetLastError();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(cut_nd.data(), nd, ncut * 4, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (nd) dev_free(nd, st);
    if (e != cudaSuccess) return cuda_status(e, "row groups");
  }
  // The wider cuts, halved until their pieces fit or are one row; only
  // those pieces are counted again.  A split cut s keeps its pieces as bits
  // of mask[s] (a piece starting at row j of the cut) and their counts at
  // sub[32 s + j].
  std::vector<int32_t> slot(ncut, -1);
  std::vector<uint32_t> mask;
  std::vector<int32_t> sub;
  std::vector<int2> pend, nextp;
  for (int64_t c = 0; c < ncut; c++) {
    const int32_t r0 = (int32_t)(c * kGroupFirstRows);
    const int32_t r1 = (int32_t)std::min<int64_t>(m, r0 + kGroupFirstRows);
    if (cut_nd[c] > kGroupCap && r1 - r0 > 1) {
      slot[c] = (int32_t)mask.size();
      mask.push_back(0u);
      const int32_t mid = r0 + (r1 - r0) / 2;
      pend.push_back(make_int2(r0, mid));
      pend.push_back(make_int2(mid, r1));
    }
  }
  sub.assign(mask.size() * kGroupFirstRows, 0);
  std::vector<int32_t> hn;
  for (int round = 1; !pend.empty(); round++) {
    if (round > 40) return set_error(EPET_ERR_INVALID, "internal: row groups unmeasured");
    const size_t n = pend.size();
    hn.resize(n);
    int2* cand = nullptr;
    int32_t* nd = nullptr;
    cudaError_t e = dev_alloc((void**)&cand, n * sizeof(int2), st);
    if (e == cudaSuccess) e = dev_alloc((void**)&nd, n * 4, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(cand, pend.data(), n * sizeof(int2), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
      k_group_distinct<<<(unsigned)n, kGroupThreads, nwords * 4, st>>>(A, cand, nwords, nd);
      note_launch();
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hn.data(), nd, n * 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (cand) dev_free(cand, st);
    if (nd) dev_free(nd, st);
    if (e != cudaSuccess) return cuda_status(e, "row groups");
    nextp.clear();
    for (size_t k = 0; k < n; k++) {
      const int2 p = pend[k];
      if (hn[k] > kGroupCap && p.y - p.x > 1) {
        const int32_t mid = p.x + (p.y - p.x) / 2;
        nextp.push_back(make_int2(p.x, mid));
        nextp.push_back(make_int2(mid, p.y));
      } else {
        const int32_t s = slot[p.x / kGroupFirstRows], j = p.x % kGroupFirstRows;
        mask[s] |= 1u << j;
        sub[(size_t)s * kGroupFirstRows + j] = hn[k];
      }
    }
    pend.swap(nextp);
  }
  // the groups in row order: the cuts kept whole, and a split cut's pieces
  out->clear();
  out->reserve(ncut + sub.size() / 8);
  int64_t tb = 0;
  for (int64_t c = 0; c < ncut; c++) {
    const int32_t r0 = (int32_t)(c * kGroupFirstRows);
    const int32_t r1 = (int32_t)std::min<int64_t>(m, r0 + kGroupFirstRows);
    uint32_t msk = slot[c] < 0 ? 1u : mask[slot[c]];
    if (!(msk & 1u)) return set_error(EPET_ERR_INVALID, "internal: row groups unmeasured");
    while (msk) {
      const int j = __builtin_ctz(msk);
      msk &= msk - 1u;
      const int32_t e = msk ? r0 + __builtin_ctz(msk) : r1;
      const int32_t ndv = slot[c] < 0 ? cut_nd[c] : sub[(size_t)slot[c] * kGroupFirstRows + j];
      const int32_t n = ndv > kGroupCap ? (ndv + 3) & ~3 : ndv;  // wide: padded like its row
      if (tb + n > INT32_MAX)
        return set_error(EPET_ERR_UNSUPPORTED, "row-group tables exceed int32");
      out->push_back(GroupDesc{r0 + j, e, (int32_t)tb, n});
      tb += n;
    }
  }
  return EPET_OK;
}

epet_status grouped_build(const RowSource& A, int64_t m, int64_t ncols, int64_t nnz,
                          int value_format, GroupedMatrix* G, cudaStream_t st) {
  (void)nnz;
  *G = GroupedMatrix{};
  G->fmt = value_format;
  G->n = ncols;
  if (!grouped_supported(ncols, m))
    return set_error(EPET_ERR_UNSUPPORTED, "grouped layout: %lld columns", (long long)ncols);
  int32_t* ftab = nullptr;  // first cuts' tables (scratch)
  auto fail = [&](epet_status rc) {
    if (ftab) dev_free(ftab, st);
    grouped_free(G, st);
    return rc;
  };
#define GALLOC(ptr, bytes)                                                        \
  do {                                                                            \
    cudaError_t e_ = dev_alloc((void**)&(ptr), std::max<size_t>((bytes), 16), st); \
    if (e_ != cudaSuccess) return fail(cuda_status(e_, "grouped allocation " #ptr)); \
  } while (0)
  const int nwords = bitmap_words(ncols);
  cudaError_t e = cudaFuncSetAttribute(k_group_tables, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)table_smem(nwords));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_group_tables, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  for (const void* k : {(const void*)k_group_mlem<0>, (const void*)k_group_mlem<1>,
                        (const void*)k_group_mlem<2>, (const void*)k_group_mlem_batch,
                        (const void*)k_group_colsum<0>, (const void*)k_group_colsum<1>,
                        (const void*)k_group_colsum<2>})
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGroupSmem);
  if (e != cudaSuccess) return fail(cuda_status(e, "grouped kernels"));
  // the padded row pointers (rows padded to whole 4-entry chunks)
  GALLOC(G->row_ptr, (m + 1) * 8);
  {
    int64_t *len = nullptr, *tmp = nullptr;
    GALLOC(len, std::max<int64_t>(m, 1) * 8);
    GALLOC(tmp, scan_tmp_elems(m) * 8);
    epet_status rc = EPET_OK;
    if (m > 0) {
      k_padded_len<<<ceil_div(m, 256), 256, 0, st>>>(A, m, len);
      note_launch();
      rc = exclusive_scan_i64(len, G->row_ptr, m, tmp, st);
    } else {
      cudaMemsetAsync(G->row_ptr, 0, 8, st);
    }
    if (rc == EPET_OK) {
      e = cudaMemcpyAsync(&G->npad, G->row_ptr + m, 8, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) rc = cuda_status(e, "padded layout");
    }
    dev_free(len, st);
    dev_free(tmp, st);
    if (rc != EPET_OK) return fail(rc);
  }
  GALLOC(G->val32, std::max<int64_t>(G->npad, 4) * 4);
  GALLOC(G->loc, std::max<int64_t>(G->npad, 4) * 2);
  // the groups; the first cuts that fit are laid out on the way
  GALLOC(ftab, ceil_div(std::max<int64_t>(m, 1), (int64_t)kGroupFirstRows) * kGroupCap * 4);
  std::vector<GroupDesc> hg;
  {
    const epet_status rc = form_groups(A, m, ncols, FirstCuts{G->row_ptr, ftab, G->val32, G->loc},
                                       &hg, st);
    if (rc != EPET_OK) return fail(rc);
  }
  G->ngroups = (int64_t)hg.size();
  G->nslots = hg.empty() ? 0 : (int64_t)hg.back().tb + hg.back().nd;
  const int64_t ns = std::max<int64_t>(G->nslots, 1);
  GALLOC(G->groups, hg.size() * sizeof(GroupDesc));
  GALLOC(G->table, ns * 4);
  GALLOC(G->partial, ns * 4);
  GALLOC(G->cg_ptr, (ncols + 1) * 8);
  if (!hg.empty()) {
    e = cudaMemcpyAsync(G->groups, hg.data(), hg.size() * sizeof(GroupDesc),
                        cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return fail(cuda_status(e, "group table"));
  }
  {
    std::vector<int32_t> wide;
    for (size_t i = 0; i < hg.size(); i++)
      if (hg[i].nd > kGroupCap) wide.push_back((int32_t)i);
    G->nwide = (int64_t)wide.size();
    G->wide_h = wide;
    if (!wide.empty()) {
      GALLOC(G->wide, wide.size() * 4);
      e = cudaMemcpyAsync(G->wide, wide.data(), wide.size() * 4, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // (the host vector goes)
      if (e != cudaSuccess) return fail(cuda_status(e, "wide groups"));
    }
  }
  // the tables at their slots and the layout of the groups split from wider cuts
  if (!hg.empty()) {
    k_group_tables<<<(unsigned)hg.size(), kGroupThreads, table_smem(nwords), st>>>(
        A, G->groups, m, nwords, G->row_ptr, G->table, ftab, nullptr, G->val32, G->loc);
    note_launch();
    if (cudaGetLastError() != cudaSuccess) return fail(set_error(EPET_ERR_CUDA, "group tables"));
  }
  dev_free(ftab, st);
  ftab = nullptr;
  // the slots of each column in group order: the column-major order of the
  // (group x column) table's entries, i.e. their positions (a wide group's
  // padding slots sit in column 0 and hold zero corrections)
  GALLOC(G->cg_slot, ns * 4);
  {
    const epet_status rc = csr_to_csc_positions(G->nslots, ncols, G->table, G->cg_ptr,
                                                reinterpret_cast<uint32_t*>(G->cg_slot), st);
    if (rc != EPET_OK) return fail(rc);
  }
  if (value_format != EPET_VALUES_FP32) {
    GALLOC(G->val16, std::max<int64_t>(G->npad, 4) * 2);
    GALLOC(G->scale, std::max<int64_t>(m, 1) * 4);
    if (m > 0) {
      if (value_format == EPET_VALUES_BF16)
        k_group_quantise<1><<<ceil_div(m * 32, 256), 256, 0, st>>>(G->row_ptr, G->val32, m,
                                                                     G->scale, G->val16);
      else
        k_group_quantise<2><<<ceil_div(m * 32, 256), 256, 0, st>>>(G->row_ptr, G->val32, m,
                                                                     G->scale, G->val16);
      note_launch();
      if (cudaGetLastError() != cudaSuccess) return fail(set_error(EPET_ERR_CUDA, "quantise"));
    }
  }
#undef GALLOC
  G->plan_cols = default_plan(ncols ? (double)G->nslots / ncols : 0.0);
  return EPET_OK;
}

static GroupIterArgs iter_args(const GroupedMatrix& G, const float* x, const float* y,
                               float* ybar) {
  return GroupIterArgs{G.groups, G.ngroups, G.row_ptr,
                       G.fmt == EPET_VALUES_FP32 ? (const void*)G.val32 : (const void*)G.val16,
                       G.scale, G.loc, G.table, x, y, ybar, G.partial};
}

size_t grouped_batch_desc_bytes() { return sizeof(GroupIterArgs); }

void grouped_batch_desc(const GroupedMatrix& G, const float* x, const float* y, float* ybar,
                        void* out) {
  *static_cast<GroupIterArgs*>(out) = iter_args(G, x, y, ybar);
}

static unsigned pass_grid(int64_t ngroups) {
  return (unsigned)std::max<int64_t>(
      1, std::min<int64_t>((ngroups + kGroupWarps - 1) / kGroupWarps, (int64_t)num_sms()));
}

epet_status grouped_pass_batch(const void* desc, const int64_t* gstart, int np,
                               int64_t total_groups, const int32_t* wide, int64_t nwide,
                               cudaStream_t st) {
  if (total_groups <= 0) return EPET_OK;
  k_group_mlem_batch<<<pass_grid(total_groups), kGroupWarps * 32, kGroupSmem, st>>>(
      static_cast<const GroupIterArgs*>(desc), gstart, np);
  EPET_LAUNCHED();
  if (nwide > 0) {
    k_group_mlem_batch_wide<<<(unsigned)ceil_div(nwide * 32, (int64_t)128), 128, 0, st>>>(
        static_cast<const GroupIterArgs*>(desc), gstart, np, wide, nwide);
    EPET_LAUNCHED();
  }
  return EPET_OK;
}

epet_status grouped_column_sums(const GroupedMatrix& G, bool quantised, float* out,
                                cudaStream_t st) {
  if (G.ngroups > 0) {
    GroupIterArgs a = iter_args(G, nullptr, nullptr, nullptr);
    int fmt = G.fmt;
    if (!quantised) {
      if (!G.val32) return set_error(EPET_ERR_INVALID, "internal: FP32 values released");
      a.val = G.val32;
      fmt = EPET_VALUES_FP32;
    }
    const unsigned grid = pass_grid(G.ngroups);
    switch (fmt) {
      case EPET_VALUES_BF16: k_group_colsum<1><<<grid, kGroupWarps * 32, kGroupSmem, st>>>(a); break;
      case EPET_VALUES_FP16: k_group_colsum<2><<<grid, kGroupWarps * 32, kGroupSmem, st>>>(a); break;
      default: k_group_colsum<0><<<grid, kGroupWarps * 32, kGroupSmem, st>>>(a);
    }
    EPET_LAUNCHED();
  }
  return launch_sums(G.plan_cols, G.cg_ptr, G.cg_slot, G.partial, G.n, EpiKeep{out},
                     nullptr, st);
}

int grouped_pass_kernels(const GroupedMatrix& G) {
  return G.ngroups == 0 ? 0 : (G.nwide > 0 ? 2 : 1);
}

epet_status grouped_pass(const GroupedMatrix& G, const float* x, const float* y, float* ybar,
                         cudaStream_t st) {
  if (G.ngroups == 0) return EPET_OK;
  const GroupIterArgs a = iter_args(G, x, y, ybar);
  const unsigned grid = pass_grid(G.ngroups);
  // (the shared-memory size was allowed when the layout was built: this
  // launch may be captured in a graph)
  switch (G.fmt) {
    case EPET_VALUES_BF16: k_group_mlem<1><<<grid, kGroupWarps * 32, kGroupSmem, st>>>(a); break;
    case EPET_VALUES_FP16: k_group_mlem<2><<<grid, kGroupWarps * 32, kGroupSmem, st>>>(a); break;
    default: k_group_mlem<0><<<grid, kGroupWarps * 32, kGroupSmem, st>>>(a);
  }
  EPET_LAUNCHED();
  if (G.nwide > 0) {
    const unsigned wgrid = (unsigned)ceil_div(G.nwide * 32, (int64_t)128);
    switch (G.fmt) {
      case EPET_VALUES_BF16: k_group_mlem_wide<1><<<wgrid, 128, 0, st>>>(a, G.wide, G.nwide); break;
      case EPET_VALUES_FP16: k_group_mlem_wide<2><<<wgrid, 128, 0, st>>>(a, G.wide, G.nwide); break;
      default: k_group_mlem_wide<0><<<wgrid, 128, 0, st>>>(a, G.wide, G.nwide);
    }
    EPET_LAUNCHED();
  }
  return EPET_OK;
}

}  // namespace epet
