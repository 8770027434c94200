// bfly.cu — fused chain kernel for Fausts whose factors all have butterfly
// supports (faust_butterfly.hpp:459-492, butterfly_support): factor S of
// size n (a power of two) with stride h stores, in row r, the two entries at
// columns r & ~h and r | h (in that order).  Rows r and r ^ h read the same
// two inputs, so a thread that holds the 2^g rows spanned by g strides can
// apply up to g consecutive factors in registers and touch shared memory
// once per g factors instead of once per factor:
//
//   pass = up to G consecutive factors (application order) with at most G
//          distinct strides; orbit = base + any subset of those strides;
//   per pass every thread loads its orbits' rows of the column tile from
//   shared memory, applies the factors in registers, stores them back (or,
//   in the last pass, to Y); one block barrier per pass.
//
// Entry order is the library's canonical one: out[r] = fma(v1, x[r|h],
// fma(v0, x[r&~h], +0)) with (v0, v1) row r's stored values in order, so the
// result is bit-identical to the per-factor CSR product.
#include <algorithm>
#include <cstdlib>
#include <cstdint>
#include <vector>

#include "csr.cuh"
#include "fgb_internal.cuh"

namespace fgb {

constexpr int BF_MAXS = 64;   // factors per chain
constexpr int BF_G = 3;       // stride slots per pass in the plan (two are used)
constexpr int BF_THREADS = 256;

struct BflyPlan {
  int n, nsteps, npasses;
  const void* val[BF_MAXS];   // step s (application order): 2 values per row
  int stride[BF_MAXS];
  int pass_first[BF_MAXS], pass_n[BF_MAXS], pass_g[BF_MAXS];
  int pass_bit[BF_MAXS][BF_G];  // orbit strides of the pass, ascending
  int step_bit[BF_MAXS];        // index of step s's stride among its pass's strides
};

template <typename T>
struct V2;
template <>
struct V2<float> {
  using type = float2;
};
template <>
struct V2<double> {
  using type = double2;
};

template <typename T, int TC>
__device__ __forceinline__ void ld_row(const T* p, T (&x)[TC]) {
  if constexpr (TC * sizeof(T) == 16) {
    if constexpr (sizeof(T) == 4) {
      const float4 v = *reinterpret_cast<const float4*>(p);
      x[0] = v.x, x[1] = v.y, x[2] = v.z, x[3] = v.w;
    } else {
      const double2 v = *reinterpret_cast<const double2*>(p);
      x[0] = v.x, x[1] = v.y;
    }
  } else {
#pragma unroll
    for (int t = 0; t < TC; ++t) x[t] = p[t];
  }
}

template <typename T, int TC>
__device__ __forceinline__ void st_row(T* p, const T (&x)[TC]) {
  if constexpr (TC * sizeof(T) == 16) {
    if constexpr (sizeof(T) == 4)
      *reinterpret_cast<float4*>(p) = make_float4(x[0], x[1], x[2], x[3]);
    else
      *reinterpret_cast<double2*>(p) = make_double2(x[0], x[1]);
  } else {
#pragma unroll
    for (int t = 0; t < TC; ++t) p[t] = x[t];
  }
}

// 16-byte row slot of matrix row r in the shared tile.  Its low three bits
// are XORed with (r3, r4, r3 ^ r4), so that the eight rows one quarter-warp
// touches (eight consecutive orbits, same position in the orbit) land in
// distinct bank groups for every pass stride pair of n = 4096 except
// (1, 8), a lone 2, and (2, 2^j) with j >= 4, which are 2-way.
__device__ __forceinline__ int bf_slot(int r) { return r ^ ((0x3650 >> (((r >> 3) & 3) << 2)) & 7); }

// One orbit of a pass with two strides (rows base, +b0, +b1, +b0+b1) or one
// stride (rows base, +b0), and the values of the pass's factors on its rows.
template <typename T>
struct BfItem {
  int row[4];
  typename V2<T>::type v[2][4];
};

template <typename T>
__device__ __forceinline__ void bf_item(const BflyPlan& p, int ps, int o, BfItem<T>& it) {
  using T2 = typename V2<T>::type;
  const int g = p.pass_g[ps], ns = p.pass_n[ps], first = p.pass_first[ps];
  const int b0 = p.pass_bit[ps][0], b1 = p.pass_bit[ps][1];
  int base = ((o & ~(b0 - 1)) << 1) | (o & (b0 - 1));
  if (g == 2) base = ((base & ~(b1 - 1)) << 1) | (base & (b1 - 1));
  it.row[0] = base;
  it.row[1] = base + b0;
  it.row[2] = base + b1;
  it.row[3] = base + b0 + b1;
  const T2* v0 = reinterpret_cast<const T2*>(p.val[first]);
  const T2* v1 = reinterpret_cast<const T2*>(p.val[first + (ns > 1 ? 1 : 0)]);
  if (g == 2) {
#pragma unroll
    for (int k = 0; k < 4; ++k) it.v[0][k] = __ldg(v0 + it.row[k]);
#pragma unroll
    for (int k = 0; k < 4; ++k) it.v[1][k] = __ldg(v1 + it.row[k]);
  } else {
    it.v[0][0] = __ldg(v0 + it.row[0]);
    it.v[0][1] = __ldg(v0 + it.row[1]);
    if (ns > 1) {
      it.v[1][0] = __ldg(v1 + it.row[0]);
      it.v[1][1] = __ldg(v1 + it.row[1]);
    }
  }
}

// One factor on the rows of an orbit: pairs (k, k | 2^b) of local rows.
template <typename T, int TC, int B>
__device__ __forceinline__ void bf_stage(T (&xs)[4][TC], const typename V2<T>::type (&v)[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if ((k >> B) & 1) continue;
    const int k1 = k | (1 << B);
#pragma unroll
    for (int t = 0; t < TC; ++t) {
      const T a = xs[k][t], c = xs[k1][t];
      xs[k][t] = fmad(v[k].y, c, fmad(v[k].x, a, T(0)));
      xs[k1][t] = fmad(v[k1].y, c, fmad(v[k1].x, a, T(0)));
    }
  }
}

// One block per column tile of TC columns, BF_THREADS threads, two strides
// per pass.  Each thread walks its (pass, orbit) items in order and loads the
// values of its next item before working on the current one, so their L2
// latency overlaps the shared-memory work (also across the pass barrier:
// values do not depend on the tile).
template <typename T, int TC>
__global__ void __launch_bounds__(BF_THREADS, sizeof(T) == 4 ? 3 : 2)
    k_bfly_chain(const __grid_constant__ BflyPlan p, const T* __restrict__ X, int ldx, int ncols, T* __restrict__ Y,
                 int ldy) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* tile = reinterpret_cast<T*>(smem_raw);  // n slots of TC values
  const int n = p.n;
  const int j0 = blockIdx.x * TC;
  const int tid = threadIdx.x;
  int nps = 0;
  while (nps < p.npasses && tid >= (n >> p.pass_g[nps])) ++nps;
  BfItem<T> nx;
  if (nps < p.npasses) bf_item<T>(p, nps, tid, nx);
  for (int r = tid; r < n; r += BF_THREADS) {
    T x[TC];
#pragma unroll
    for (int t = 0; t < TC; ++t) x[t] = (j0 + t < ncols) ? X[r + (long)(j0 + t) * ldx] : T(0);
    st_row<T, TC>(tile + (long)bf_slot(r) * TC, x);
  }
  __syncthreads();
  for (int ps = 0; ps < p.npasses; ++ps) {
    const int g = p.pass_g[ps], ns = p.pass_n[ps], first = p.pass_first[ps];
    const bool last = ps + 1 == p.npasses;
    const int orbits = n >> g;
    const int sb0 = p.step_bit[first], sb1 = p.step_bit[first + (ns > 1 ? 1 : 0)];
    for (int o = tid; o < orbits; o += BF_THREADS) {
      const BfItem<T> it = nx;
      {
        int qo = o + BF_THREADS, qp = ps;
        if (qo >= orbits) {
          qp = ps + 1;
          qo = tid;
          while (qp < p.npasses && tid >= (n >> p.pass_g[qp])) ++qp;
        }
        if (qp < p.npasses) bf_item<T>(p, qp, qo, nx);
      }
      T xs[4][TC];
      if (g == 2) {
#pragma unroll
        for (int k = 0; k < 4; ++k) ld_row<T, TC>(tile + (long)bf_slot(it.row[k]) * TC, xs[k]);
        if (sb0 == 0) bf_stage<T, TC, 0>(xs, it.v[0]);
        else bf_stage<T, TC, 1>(xs, it.v[0]);
        if (ns > 1) {
          if (sb1 == 0) bf_stage<T, TC, 0>(xs, it.v[1]);
          else bf_stage<T, TC, 1>(xs, it.v[1]);
        }
      } else {
        // one stride: local rows 0 and 1 only
#pragma unroll
        for (int k = 0; k < 2; ++k) ld_row<T, TC>(tile + (long)bf_slot(it.row[k]) * TC, xs[k]);
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          if (s >= ns) break;
#pragma unroll
          for (int t = 0; t < TC; ++t) {
            const T a = xs[0][t], c = xs[1][t];
            xs[0][t] = fmad(it.v[s][0].y, c, fmad(it.v[s][0].x, a, T(0)));
            xs[1][t] = fmad(it.v[s][1].y, c, fmad(it.v[s][1].x, a, T(0)));
          }
        }
      }
      const int kn = g == 2 ? 4 : 2;
      if (last) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (k >= kn) continue;
#pragma unroll
          for (int t = 0; t < TC; ++t)
            if (j0 + t < ncols) Y[it.row[k] + (long)(j0 + t) * ldy] = xs[k][t];
        }
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k)
          if (k < kn) st_row<T, TC>(tile + (long)bf_slot(it.row[k]) * TC, xs[k]);
      }
    }
    if (!last) __syncthreads();
  }
}

// ------------------------------------------------------------------ two phases
// For chains whose application order first uses only strides below 2^a and
// then only strides of 2^a and above (the order of butterfly_support's
// factors applied right to left), the rows split as r = q * 2^a + p: the
// first phase only mixes rows of the same block q (in-block index p), the
// second only rows of the same p (index q).  Each phase is a run of small
// independent groups of rows, so a CTA owns a few groups, keeps their factor
// values in shared memory once, and streams column tiles past them -- the
// factor values are read once per CTA instead of once per column tile.
// Between the phases the intermediate Z is stored block-transposed
// (position p * (n / 2^a) + q), so both phases read and write their groups as
// contiguous runs; the columns go in chunks whose Z stays in L2.  Entry
// order per factor is the canonical one, so results equal the CSR chain's.
//
// In one phase: groups of S rows (in-group index i), NG groups; a CTA owns
// BP_GPC consecutive groups and steps over tiles of BP_NT x 4 columns.  The
// phase input holds group g's rows at positions g * S + i, the output at
// i * NG + g; the factor values of (g, i) sit at row g * S + i (first phase)
// or i * NG + g (second phase).  Orbits of 8 rows (three strides of the
// in-group index) x 4 columns per thread, up to three factors per pass.
constexpr int BP_GPC = 8;     // groups per CTA
constexpr int BP_NT = 4;      // 4-column tiles per CTA step
constexpr int BP_MAXF = 8;    // factors per phase
constexpr int BP_MAXP = 8;    // passes per phase

struct BflyPhase {
  int ng;        // groups of the phase (n / S)
  int vmode;     // 0: value row g * S + i; 1: value row i * ng + g
  int nf, npasses;
  const float* val[BP_MAXF];    // 2 values per row, application order
  int lbit[BP_MAXF];            // stride of factor f as a bit of the in-group index
  int pass_first[BP_MAXP], pass_n[BP_MAXP];
  int pass_pos[BP_MAXP][3];     // orbit span bits of the pass, ascending
  int pass_local[BP_MAXF];      // factor f's bit among its pass's span (0..2)
};

// Local row R = i * BP_GPC + g of the CTA's groups, 16-byte slot with bits
// 0-2 XORed with bits 3-5: conflict-free for eight consecutive groups at one
// in-group row (the passes, the stores) and for eight consecutive in-group
// rows of one group (the tile loads).
__device__ __forceinline__ int bp_slot(int R) { return R ^ ((R >> 3) & 7); }

template <int B>
__device__ __forceinline__ void bp_stage(float4 (&xs)[8], const float2 (&v)[8]) {
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    if ((k >> B) & 1) continue;
    const int k1 = k | (1 << B);
    const float2 va = v[k], vb = v[k1];
    const float4 a = xs[k], c = xs[k1];
    xs[k] = make_float4(fmad(va.y, c.x, fmad(va.x, a.x, 0.f)), fmad(va.y, c.y, fmad(va.x, a.y, 0.f)),
                        fmad(va.y, c.z, fmad(va.x, a.z, 0.f)), fmad(va.y, c.w, fmad(va.x, a.w, 0.f)));
    xs[k1] = make_float4(fmad(vb.y, c.x, fmad(vb.x, a.x, 0.f)), fmad(vb.y, c.y, fmad(vb.x, a.y, 0.f)),
                         fmad(vb.y, c.z, fmad(vb.x, a.z, 0.f)), fmad(vb.y, c.w, fmad(vb.x, a.w, 0.f)));
  }
}

template <int S>
__global__ void __launch_bounds__(BP_NT * BP_GPC * S / 8, S == 64 ? 3 : 1)
    k_bfly_phase(const __grid_constant__ BflyPhase P, const float* __restrict__ in, long ld_in,
                 float* __restrict__ out, long ld_out, int ncols) {
  constexpr int ROWS = BP_GPC * S;          // rows of the CTA
  constexpr int NT = BP_NT * BP_GPC * S / 8;  // threads: one orbit x 4 columns each
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float4* tiles = reinterpret_cast<float4*>(smem_raw);                  // [BP_NT][ROWS]
  float2* vs = reinterpret_cast<float2*>(smem_raw + sizeof(float4) * BP_NT * ROWS);  // [nf][ROWS]
  const int tid = threadIdx.x;
  const int g0 = blockIdx.x * BP_GPC;
  // the CTA's factor values, once
  for (int f = 0; f < P.nf; ++f) {
    const float2* v = reinterpret_cast<const float2*>(P.val[f]);
    for (int R = tid; R < ROWS; R += NT) {
      const int g = R % BP_GPC, i = R / BP_GPC;
      const long r = P.vmode ? (long)i * P.ng + g0 + g : (long)(g0 + g) * S + i;
      vs[f * ROWS + bp_slot(R)] = __ldg(v + r);
    }
  }
  // this thread's orbit: 4-column tile tt, group g, orbit o of the group
  const int tt = tid / (ROWS / 8), rem = tid % (ROWS / 8);
  const int g = rem % BP_GPC, o = rem / BP_GPC;
  const long in0 = (long)g0 * S;
  for (long j0 = (long)blockIdx.y * BP_NT * 4; j0 < ncols; j0 += (long)gridDim.y * BP_NT * 4) {
    __syncthreads();  // values stored; previous tile consumed
    // tiles: group rows are contiguous in the input (positions g * S + i)
    for (int idx = tid; idx < BP_NT * ROWS; idx += NT) {
      const int t = idx / ROWS, Rin = idx % ROWS;
      const int gg = Rin / S, i = Rin % S;
      const long j = j0 + t * 4;
      const float* src = in + in0 + Rin + j * ld_in;
      float4 x;
      x.x = j < ncols ? src[0] : 0.f;
      x.y = j + 1 < ncols ? src[ld_in] : 0.f;
      x.z = j + 2 < ncols ? src[2 * ld_in] : 0.f;
      x.w = j + 3 < ncols ? src[3 * ld_in] : 0.f;
      tiles[t * ROWS + bp_slot(i * BP_GPC + gg)] = x;
    }
    __syncthreads();
    float4* tile = tiles + tt * ROWS;
    for (int ps = 0; ps < P.npasses; ++ps) {
      const bool last = ps + 1 == P.npasses;
      const int p0 = P.pass_pos[ps][0], p1 = P.pass_pos[ps][1], p2 = P.pass_pos[ps][2];
      int base = o;
      base = ((base >> p0) << (p0 + 1)) | (base & ((1 << p0) - 1));
      base = ((base >> p1) << (p1 + 1)) | (base & ((1 << p1) - 1));
      base = ((base >> p2) << (p2 + 1)) | (base & ((1 << p2) - 1));
      int R[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        R[k] = (base + ((k & 1) << p0) + (((k >> 1) & 1) << p1) + (((k >> 2) & 1) << p2)) * BP_GPC + g;
      float4 xs[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) xs[k] = tile[bp_slot(R[k])];
      const int first = P.pass_first[ps], nfp = P.pass_n[ps];
      for (int f = first; f < first + nfp; ++f) {
        const float2* vf = vs + f * ROWS;
        float2 v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = vf[bp_slot(R[k])];
        const int b = P.pass_local[f];
        if (b == 0) bp_stage<0>(xs, v);
        else if (b == 1) bp_stage<1>(xs, v);
        else bp_stage<2>(xs, v);
      }
      if (last) {
        // output position i * ng + g: eight consecutive groups are one
        // 32-byte run per column
        const long j = j0 + tt * 4;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          const int i = R[k] / BP_GPC;
          float* dst = out + (long)i * P.ng + g0 + g + j * ld_out;
          if (j < ncols) dst[0] = xs[k].x;
          if (j + 1 < ncols) dst[ld_out] = xs[k].y;
          if (j + 2 < ncols) dst[2 * ld_out] = xs[k].z;
          if (j + 3 < ncols) dst[3 * ld_out] = xs[k].w;
        }
      } else {
#pragma unroll
        for (int k = 0; k < 8; ++k) tile[bp_slot(R[k])] = xs[k];
        __syncthreads();
      }
    }
  }
}

// Plan of one phase: factors (application order) first..first+cnt, strides
// as bits of the phase's in-group index (stride bit - shift); passes of up to
// three distinct bits, padded with the lowest unused ones.
static bool build_phase(const std::vector<const float*>& vals, const std::vector<int>& bits, int first, int cnt,
                        int shift, int slog, int ng, int vmode, BflyPhase& P) {
  if (cnt > BP_MAXF || slog < 3) return false;
  P.ng = ng;
  P.vmode = vmode;
  P.nf = cnt;
  P.npasses = 0;
  for (int u = 0; u < cnt; ++u) {
    P.val[u] = vals[first + u];
    P.lbit[u] = bits[first + u] - shift;
  }
  for (int s = 0; s < cnt;) {
    if (P.npasses == BP_MAXP) return false;
    const int ps = P.npasses++;
    std::vector<int> pos;
    int e = s;
    while (e < cnt) {
      const bool have = std::find(pos.begin(), pos.end(), P.lbit[e]) != pos.end();
      if (!have && (int)pos.size() == 3) break;
      if (!have) pos.push_back(P.lbit[e]);
      ++e;
    }
    for (int b = 0; (int)pos.size() < 3 && b < slog; ++b)
      if (std::find(pos.begin(), pos.end(), b) == pos.end()) pos.push_back(b);
    std::sort(pos.begin(), pos.end());
    P.pass_first[ps] = s;
    P.pass_n[ps] = e - s;
    for (int q = 0; q < 3; ++q) P.pass_pos[ps][q] = pos[q];
    for (int u = s; u < e; ++u) P.pass_local[u] = (int)(std::find(pos.begin(), pos.end(), P.lbit[u]) - pos.begin());
    s = e;
  }
  return true;
}

template <int S>
static fgb_status launch_phase(fgb_ctx* ctx, const BflyPhase& P, const float* in, long ld_in, float* out,
                               long ld_out, int ncols) {
  constexpr int ROWS = BP_GPC * S;
  const size_t smem = sizeof(float4) * BP_NT * ROWS + sizeof(float2) * (size_t)P.nf * ROWS;
  auto kern = k_bfly_phase<S>;
  if (smem > 48 * 1024)
    FGB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  // column steps of the chunk spread evenly over about one wave of CTAs
  const int steps = (ncols + BP_NT * 4 - 1) / (BP_NT * 4);
  const int ymax = std::max(1, (int)(3L * ctx->sm_count * BP_GPC / P.ng));
  const int spc = (steps + ymax - 1) / ymax;
  dim3 grid(P.ng / BP_GPC, (steps + spc - 1) / spc);
  kern<<<grid, BP_NT * ROWS / 8, smem, ctx->stream>>>(P, in, ld_in, out, ld_out, ncols);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

static fgb_status launch_phase_s(fgb_ctx* ctx, int slog, const BflyPhase& P, const float* in, long ld_in,
                                 float* out, long ld_out, int ncols) {
  if (slog == 5) return launch_phase<32>(ctx, P, in, ld_in, out, ld_out, ncols);
  if (slog == 6) return launch_phase<64>(ctx, P, in, ld_in, out, ld_out, ncols);
  return launch_phase<128>(ctx, P, in, ld_in, out, ld_out, ncols);
}

// The two-phase chain when the application order allows it (FP32, forward
// split of the strides, group sizes 32, 64 or 128); *ran tells whether it ran.
static fgb_status bfly_two_phase(fgb_faust* F, char op, int nfac, const float* X, int ldx, int ncols, float* Y,
                                 int ldy, bool* ran) {
  *ran = false;
  fgb_ctx* ctx = F->ctx;
  const int J = (int)F->f.size();
  const int n = F->f[0].rows;
  int m = 0;
  while ((1 << m) < n) ++m;
  std::vector<const float*> vals(nfac);
  std::vector<int> bits(nfac);
  for (int s = 0; s < nfac; ++s) {
    const int q = nfac - 1 - s;
    const DevFactor& f = F->f[op == 'N' ? q : J - 1 - q];
    vals[s] = (const float*)(op == 'N' ? f.val : f.t_val);
    int b = 0;
    while ((1 << b) < f.bfly) ++b;
    bits[s] = b;
  }
  // split point: prefix bits all < a <= suffix bits, a as close to m / 2 as
  // the order allows, both group sizes 32..128
  int best_a = -1, best_L = -1;
  for (int L = 1; L < nfac; ++L) {
    int mx = 0, mn = m;
    for (int s = 0; s < L; ++s) mx = std::max(mx, bits[s]);
    for (int s = L; s < nfac; ++s) mn = std::min(mn, bits[s]);
    for (int a = mx + 1; a <= mn; ++a)
      if (a >= 5 && a <= 7 && m - a >= 5 && m - a <= 7 && (best_a < 0 || std::abs(2 * a - m) < std::abs(2 * best_a - m)))
        best_a = a, best_L = L;
  }
  if (best_a < 0) return FGB_OK;
  const int a = best_a, L = best_L;
  const int SA = 1 << a, SB = n >> a;
  BflyPhase PA, PB;
  if (!build_phase(vals, bits, 0, L, 0, a, n / SA, 0, PA)) return FGB_OK;
  if (!build_phase(vals, bits, L, nfac - L, a, m - a, SA, 1, PB)) return FGB_OK;
  // column chunks whose intermediate (n x cw FP32) stays in L2
  const long zcap = 32L << 20;
  long cw = std::max<long>(BP_NT * 4, (zcap / ((long)n * 4)) / (BP_NT * 4) * (BP_NT * 4));
  cw = std::min<long>(cw, ncols);
  const size_t need = (size_t)n * cw * sizeof(float);
  if (F->bz_bytes < need) {
    dfree(F->bz);
    F->bz = nullptr;
    F->bz_bytes = 0;
    FGB_TRY(dmalloc(ctx, &F->bz, need));
    F->bz_bytes = need;
  }
  float* Z = (float*)F->bz;
  *ran = true;
  for (long c0 = 0; c0 < ncols; c0 += cw) {
    const int w = (int)std::min<long>(cw, ncols - c0);
    FGB_TRY(launch_phase_s(ctx, a, PA, X + c0 * ldx, ldx, Z, n, w));
    FGB_TRY(launch_phase_s(ctx, m - a, PB, Z, n, Y + c0 * ldy, ldy, w));
  }
  return FGB_OK;
}

// ------------------------------------------------------------------ detection
// bad[q] = 1 unless factor q is a butterfly factor of stride h[q].
__global__ void k_bfly_detect(const int* __restrict__ rowptr, const int* __restrict__ colind, int n,
                              int* __restrict__ bad, int* __restrict__ hout) {
  const int h = colind[1] - colind[0];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *hout = h;
    if (h <= 0 || h >= n || (h & (h - 1)) || rowptr[n] != 2 * n) *bad = 1;
  }
  if (h <= 0 || h >= n) return;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    if (rowptr[r] != 2 * r || colind[2 * r] != (r & ~h) || colind[2 * r + 1] != (r | h)) *bad = 1;
  }
}

// Caches DevFactor::bfly (stride, or 0) for every factor of F.
static fgb_status bfly_detect(fgb_faust* F) {
  fgb_ctx* ctx = F->ctx;
  const int J = (int)F->f.size();
  bool need = false;
  for (auto& f : F->f) need = need || f.bfly < 0;
  if (!need) return FGB_OK;
  std::vector<int> cand(J, 0);
  int ncand = 0;
  for (int q = 0; q < J; ++q) {
    const DevFactor& f = F->f[q];
    const bool shape = f.format == FGB_CSR && f.rows == f.cols && f.rows >= 2 && (f.rows & (f.rows - 1)) == 0 &&
                       f.nnz == 2 * f.rows;
    cand[q] = shape;
    ncand += shape;
  }
  if (ncand) {
    int* d = nullptr;
    FGB_TRY(dmalloc(ctx, (void**)&d, sizeof(int) * 2 * J));
    FGB_CUDA(ctx, cudaMemsetAsync(d, 0, sizeof(int) * 2 * J, ctx->stream));
    for (int q = 0; q < J; ++q) {
      if (!cand[q]) continue;
      const DevFactor& f = F->f[q];
      const int g = std::max(1, std::min(2 * ctx->sm_count, (f.rows + 255) / 256));
      k_bfly_detect<<<g, 256, 0, ctx->stream>>>(f.rowptr, f.colind, f.rows, d + q, d + J + q);
      FGB_LAUNCHED(ctx);
    }
    std::vector<int> h(2 * J);
    cudaError_t e = cudaMemcpyAsync(h.data(), d, sizeof(int) * 2 * J, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    dfree(d);
    if (e != cudaSuccess) return cuda_check(ctx, e, "butterfly detection");
    for (int q = 0; q < J; ++q) F->f[q].bfly = (cand[q] && !h[q]) ? h[J + q] : 0;
  } else {
    for (auto& f : F->f) f.bfly = 0;
  }
  return FGB_OK;
}

// Passes of at most two consecutive factors (application order) with at most
// two distinct strides.
static void build_plan(fgb_faust* F, char op, int nfac, BflyPlan& p) {
  const int J = (int)F->f.size();
  p.n = F->f[0].rows;
  p.nsteps = nfac;
  // application order: G_{nfac-1} first, with G_q = S_q (op N) or S_{J-1-q}^T
  for (int s = 0; s < nfac; ++s) {
    const int q = nfac - 1 - s;
    const DevFactor& f = F->f[op == 'N' ? q : J - 1 - q];
    p.val[s] = op == 'N' ? f.val : f.t_val;
    p.stride[s] = f.bfly;
  }
  p.npasses = 0;
  for (int s = 0; s < nfac;) {
    const int ps = p.npasses++;
    const int cnt = (s + 1 < nfac) ? 2 : 1;
    int bits[2] = {p.stride[s], cnt > 1 ? p.stride[s + 1] : 0};
    int nb = (cnt > 1 && bits[1] != bits[0]) ? 2 : 1;
    if (nb == 2 && bits[1] < bits[0]) std::swap(bits[0], bits[1]);
    p.pass_first[ps] = s;
    p.pass_n[ps] = cnt;
    p.pass_g[ps] = nb;
    p.pass_bit[ps][0] = bits[0];
    p.pass_bit[ps][1] = nb == 2 ? bits[1] : 0;
    p.pass_bit[ps][2] = 0;
    for (int u = 0; u < cnt; ++u) p.step_bit[s + u] = p.stride[s + u] == bits[0] ? 0 : 1;
    s += cnt;
  }
}

template <typename T, int TC>
static fgb_status launch_bfly(fgb_faust* F, char op, int nfac, const T* X, int ldx, int ncols, T* Y, int ldy) {
  fgb_ctx* ctx = F->ctx;
  BflyPlan p;
  build_plan(F, op, nfac, p);
  const size_t smem = (size_t)p.n * TC * sizeof(T);
  auto kern = k_bfly_chain<T, TC>;
  if (smem > 48 * 1024)
    FGB_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int tiles = (ncols + TC - 1) / TC;
  kern<<<tiles, BF_THREADS, smem, ctx->stream>>>(p, X, ldx, ncols, Y, ldy);
  FGB_LAUNCHED(ctx);
  return FGB_OK;
}

// Runs G_0 ... G_{nfac-1} X with the butterfly kernel when every factor of the
// chain is a butterfly factor and the column tile fits in shared memory;
// *ran tells whether it did.  force: also for few column tiles.
fgb_status bfly_chain(fgb_faust* F, char op, int nfac, const void* X, int ldx, int ncols, void* Y, int ldy,
                      bool force, bool* ran) {
  *ran = false;
  fgb_ctx* ctx = F->ctx;
  if (F->dtype != FGB_F32 && F->dtype != FGB_F64) return FGB_OK;
  if (nfac < 1 || nfac > BF_MAXS || ncols <= 0) return FGB_OK;
  FGB_TRY(bfly_detect(F));
  const int J = (int)F->f.size();
  for (int q = 0; q < nfac; ++q)
    if (F->f[op == 'N' ? q : J - 1 - q].bfly <= 0) return FGB_OK;
  const int n = F->f[0].rows;
  for (auto& f : F->f)
    if (f.rows != n) return FGB_OK;
  for (int q = 0; q < nfac; ++q) {
    const DevFactor& f = F->f[op == 'N' ? q : J - 1 - q];
    if (op != 'N' && !f.has_t) return FGB_OK;
    // pairs of values are read as one 2-element vector
    if ((uintptr_t)(op == 'N' ? f.val : f.t_val) % (2 * dtype_size(F->dtype))) return FGB_OK;
  }
  const size_t cap = std::min<size_t>(ctx->smem_optin ? ctx->smem_optin : 227 * 1024, 200 * 1024);
  if ((size_t)n * 16 > cap) return FGB_OK;  // one 16-byte row per matrix row
  const int tc = 16 / (int)dtype_size(F->dtype);
  const long tiles = (ncols + tc - 1) / tc;
  if (!force && tiles < ctx->sm_count) return FGB_OK;
  if (F->dtype == FGB_F32 && !getenv("FGB_BFLY_ONE_PHASE")) {
    FGB_TRY(bfly_two_phase(F, op, nfac, (const float*)X, ldx, ncols, (float*)Y, ldy, ran));
    if (*ran) return FGB_OK;
  }
  *ran = true;
  if (F->dtype == FGB_F32)
    return launch_bfly<float, 4>(F, op, nfac, (const float*)X, ldx, ncols, (float*)Y, ldy);
  return launch_bfly<double, 2>(F, op, nfac, (const double*)X, ldx, ncols, (double*)Y, ldy);
}

}  // namespace fgb
