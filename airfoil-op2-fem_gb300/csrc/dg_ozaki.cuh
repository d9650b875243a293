// Element-kernel contraction on the tensor cores (fp16 digit operands), exact to FP64 accuracy (included by
// dg_solver.cu inside namespace dg).
//
// On GB300 the FP64 pipe issues about 2 DFMA lanes per clock per SM, while mma.sync on 16-bit
// operands runs at ~600 TFLOP/s with FP32 accumulation.  The even/odd contraction of the
// element kernel, Y_p = S_p X_p for the even (p = 0) and odd (p = 1) halves (rows of the operator
// S_p, columns of X_p = one (cell, variable) over the staged slots), is therefore done as an
// integer product in the manner of Ozaki's error-free splitting (Ozaki, Ogita, Oishi, Rump,
// "Error-free transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59, 2012):
//
//  * every column of X_p (16 or 32 values) is scaled by its largest binary exponent E, so each
//    value is x = m 2^(E-55) with m an integer, |m| < 2^56 (the bits below 2^(E-55) are cut);
//    every operator row by its own F likewise (done once on the host).  In the element kernel
//    oz_prep does this once per staged value and forms the even/odd sums and differences exactly
//    from values aligned to 2^(E-54).  m is written in base 256 as seven signed digits d_0..d_6
//    (|d| <= 255, all with the sign of x), each exact in fp16 (the mma operands).
//  * digit products d_j c_s with j + s = L are summed into one FP32 accumulator per level L
//    (L = 0..6; the levels L >= 7 lie below 2^-56 of the leading term and are dropped).  A level
//    sums at most 7 pairs x 32 slots x 255^2 < 2^24, so every accumulation is an exact integer
//    (checked on the GPU: bit-exact against 64-bit integer sums up to 1.46e7).
//  * the seven level sums are joined as integers, T = sum_L lev_L 256^(6-L) (two 64-bit parts,
//    below 2^41 and 2^49), and T 2^(E+F-62) is rounded to the nearest double with integer instructions
//    only (oz_round; no FP64 instruction and no int-to-double conversion, which takes several
//    FP64 issue slots on this part).  The result is the correctly rounded dot product of the
//    56-bit truncations:
//    its error is below 2^-55 max|x| sum|s|, under the FP64 dot product's own error bound.
//
// Units of work: parity x 8 groups of 4 cells (x 4 variables) = 16 m16n8k16 row tiles per
// 32-cell tile; each needs 28 mma per k-step of 16 slots.  Non-finite inputs in a column give NaN.
// Each row tile takes the operator rows 8 at a time (one n-tile of mma).

// Tables of the operator blocks S_p (T = 0: rows of S_p are the outputs, the element kernel),
// of their transposes (T = 1: columns of S_p are the outputs, the adjoint element kernel) and of
// the dense rows A = [Drw | Dsw | -LIFT/2] (T = 2, parity 0 only: the element kernel's dense form).
constexpr int kOzRows = 32;  // outputs per parity: up to 4 n-tiles of 8
constexpr int kOzTables = 3;
__constant__ int c_ozf[kOzTables][7][2][kOzRows];  // biased binary exponent F of every output row: T, order, parity, row
__device__ uint2 g_ozb[kOzTables][7][2][4][7][2][32];  // B fragments: T, order, parity, n-tile, digit s, k-step, lane

// Orders that use the even/odd blocks on the tensor cores: N = 3, 4, 5 (steps on the K=32768
// O-grid, first form: 365 -> 328, 564 -> 477, 909 -> 720 us).  At N = 1 and 2 the even/odd blocks
// were too small a share of the element kernel for the split to pay (N = 1: 184 -> 192 us, N = 2:
// 236 -> 252 us); those orders use the dense rows instead (ozd_used).  Orders up to 5 fit the
// exactness bound (at most two k-steps of 16 slots); N = 6 needs three.
constexpr int kOzMaxN = 5;
constexpr bool oz_used(int N, bool tc) { return tc && (N == 3 || N == 4 || N == 5); }
// The adjoint element kernel's transposed contraction: N = 3 (the transposed blocks of N = 4
// need six n-tiles of outputs).
constexpr bool oz_used_t(int N, bool tc) { return tc && N == 3; }
// Minimum resident blocks per SM for the element kernel's register allocation in this form.
constexpr int oz_min_blocks(int N) { return N <= 3 ? 3 : (N == 4 ? 2 : 1); }
// The dense form (element-kernel form 3 at N = 1, 2): the NK = 2 Np + 3 Nfp staged slots of every
// column go through the dense rows A directly, without the even/odd butterfly and the
// recombination of the outputs, at twice the mma count of the even/odd blocks.  On the K=32768
// O-grid: steps 187 -> 175 us (N = 1) and 241 -> 222 us (N = 2).  At N = 3 (NK = 32, still within
// two k-steps) it measured slower than the even/odd blocks on the tensor cores (341 vs 327 us:
// each warp's share of the contraction doubles, and spills rise), so N = 3 keeps those.
constexpr bool ozd_used(int N, int mode) { return mode == 2 && N >= 1 && N <= 2; }
// Minimum resident blocks per SM of an element kernel of form TC (0 FP64, 1 even/odd blocks on the
// tensor cores, 2 dense rows on the tensor cores) at order N.
constexpr int elem_min_blocks(int N, int TC) {
  return (ozd_used(N, TC) || oz_used(N, TC != 0)) ? oz_min_blocks(N) : 1;
}

__device__ __forceinline__ void mma_f16_16816(float c[4], const uint32_t a[4], const uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// Digit j (0 = most significant) of the magnitudes (hi:lo, < 2^56) of two values, low k first,
// as an fp16 pair with the values' signs (v = 0x64006400 | signs, bit 15 the low value's, bit 31
// the high value's): one byte permute puts byte (6 - j) of each magnitude into the mantissa of
// the fp16 1024 (bits 0x6400 | d), the mask and v keep those bytes and add the signs, and
// subtracting v (+-1024 in each half) leaves exactly +-d (|d| <= 255).  Three instructions per
// pair of digits (as two floats made from the bytes and packed: six).
__device__ __forceinline__ uint32_t oz_pair(const uint32_t hl, const uint32_t ll, const uint32_t hh,
                                            const uint32_t lh, const int j, const uint32_t v) {
  const uint32_t wl = j < 3 ? hl : ll, wh = j < 3 ? hh : lh;
  const uint32_t b = j < 3 ? (uint32_t)(2 - j) : (uint32_t)(6 - j);
  const uint32_t r = (__byte_perm(wl, wh, b | ((4u + b) << 8)) & 0x00FF00FFu) | v;
  uint32_t out;
  asm("sub.rn.f16x2 %0, %1, %2;" : "=r"(out) : "r"(r), "r"(v));
  return out;
}

// (th 2^32 + tl) 2^sc rounded to the nearest double (ties to even), with integer instructions only:
// on this part an FP64 add holds the FP64 pipe for 16 clocks per warp, an integer instruction
// for 1/2.  With level sums below 2^24, |th| < 2^41 and |tl| < 2^49, so |T| < 2^74; for
// -1022 <= sc <= 900 the result is a normal double (its biased exponent is sc + 1022 plus the
// bit length of T, at most 1997), so no subnormal or overflow case arises.  The result equals
// RN(th 2^(32+sc) + tl 2^sc), the sum of the two exact parts rounded once.
// Host and device alike (the host copy serves the library's rounding check, dg_tc_round).
__host__ __device__ __forceinline__ int oz_clz64(const unsigned long long x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}
__host__ __device__ __forceinline__ double oz_double(const unsigned long long b) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)b);
#else
  double d;
  std::memcpy(&d, &b, sizeof d);
  return d;
#endif
}

__host__ __device__ __forceinline__ double oz_round(const long long th, const long long tl, const int sc) {
  // T = H 2^32 + L with 0 <= L < 2^32, then |T| = MH 2^32 + ML (MH < 2^42, ML < 2^32)
  const long long H = th + (tl >> 32);
  const unsigned long long L = (unsigned long long)tl & 0xFFFFFFFFull;
  const unsigned long long sign = H < 0 ? 0x8000000000000000ull : 0ull;
  unsigned long long MH, ML;
  if (H < 0) {
    MH = (unsigned long long)(-H) - (L ? 1ull : 0ull);
    ML = L ? 0x100000000ull - L : 0ull;
  } else {
    MH = (unsigned long long)H;
    ML = L;
  }
  // the leading bits in one 64-bit word S = |T| / 2^off; below 2^63 exactly (off = 0), else the
  // 10 dropped bits of ML only decide ties (sticky)
  unsigned long long S;
  int off;
  bool sticky;
  if (MH >> 31) {
    S = (MH << 22) | (ML >> 10);
    off = 10;
    sticky = (ML & 0x3FFull) != 0ull;
  } else {
    S = (MH << 32) | ML;
    off = 0;
    sticky = false;
  }
  if (S == 0ull) return 0.0;
  const int nb = 64 - oz_clz64(S);  // bit length of S
  unsigned long long q;  // significand, 2^52 <= q < 2^53
  int e2;                // value = q 2^(e2 + sc)
  if (nb <= 53) {        // (off = 0 here: S >= 2^53 otherwise)
    q = S << (53 - nb);
    e2 = nb - 53;
  } else {
    const int sh = nb - 53;
    q = S >> sh;
    const unsigned long long rem = S & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (sticky || (q & 1ull)))) q++;
    e2 = sh + off;
    if (q >> 53) {  // rounded up to 2^53
      q >>= 1;
      e2++;
    }
  }
  const unsigned long long be = (unsigned long long)(e2 + sc + 52 + 1023);
  return oz_double(sign | (be << 52) | (q & 0xFFFFFFFFFFFFFull));
}

// Bit pattern of a double -> its magnitude aligned to the biased column exponent em as an integer,
// M 2^(e - em + SH) (M the 53-bit significand), with the double's sign; 0 below 2^-63 of the
// column's leading bit.
template <int SH>
__device__ __forceinline__ long long oz_align(const unsigned long long b, const int em) {
  const int e = (int)((b >> 52) & 0x7FF);
  const unsigned long long M = e ? ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : 0ull;
  const int sh = e - em + SH;
  const unsigned long long m = sh >= 0 ? (M << sh) : (sh > -64 ? (M >> -sh) : 0ull);
  return (b >> 63) ? -(long long)m : (long long)m;
}

// One 16-row tile: cells c0..c0+3 x the four variables (row r: cell c0 + r / 4, variable r % 4, so
// the eight row lanes of a fragment read eight consecutive doubles), slots SLOT0..SLOT0+K-1
// (K <= 16 KST), times operator rows 8 NT .. 8 NT + 7 (of R) of parity P, written to Y rows
// YROW0 + row.  The k-steps are taken one after the other (their values re-read from shared
// memory) so that only one k-step's magnitudes are live next to the seven accumulators.
// XST: doubles from one slot (or output row) to the next in Xd and Yd (128 = 32 cells x 4
// variables, plus any padding).
// PRE: the slots hold operands already aligned by oz_prep (sign in bit 63, magnitude below 2^56,
// aligned to 2^(E-54)) and Ems[col] their column exponent E; otherwise the slots hold doubles,
// aligned here to 2^(E-55).
template <int T, int NORD, int K, int R, int SLOT0, int YROW0, int KST, int P, int NT, bool PRE = false,
          int XST = 128>
__device__ __forceinline__ void oz_tile(const double *__restrict__ Xd, double *__restrict__ Yd, const int c0,
                                        const int lane, const int *__restrict__ Ems = nullptr) {
  static_assert(KST <= 2 && K <= 16 * KST && R > 8 * NT && NT < 4, "four n-tiles, two k-steps at most");
  constexpr int SH = PRE ? 2 : 3;  // the alignment shift (oz_align)
  const int g = lane >> 2, t = lane & 3;
  const int col = c0 * 4 + g;  // (cell, variable) of row g; row g + 8 is col + 8
  const uint32_t *Xw = reinterpret_cast<const uint32_t *>(Xd);
  // largest binary exponent of each of the two columns over all values read (high words only)
  int em[2] = {0, 0};
  if constexpr (PRE) {
    em[0] = Ems[col];
    em[1] = Ems[col + 8];
  } else {
#pragma unroll
    for (int ks = 0; ks < KST; ks++)
#pragma unroll
      for (int r = 0; r < 2; r++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const int k = 16 * ks + 2 * t + (q & 1) + ((q >> 1) << 3);
          if (k < K) em[r] = max(em[r], (int)((Xw[2 * ((SLOT0 + k) * XST + col + 8 * r) + 1] >> 20) & 0x7FF));
        }
#pragma unroll
    for (int r = 0; r < 2; r++) {
      em[r] = max(em[r], __shfl_xor_sync(0xffffffffu, em[r], 1));
      em[r] = max(em[r], __shfl_xor_sync(0xffffffffu, em[r], 2));
    }
  }
  const uint2 *bfr = &g_ozb[T][NORD][P][NT][0][0][lane];
  float acc[7][4];
#pragma unroll
  for (int l = 0; l < 7; l++) acc[l][0] = acc[l][1] = acc[l][2] = acc[l][3] = 0.0f;
#pragma unroll
  for (int ks = 0; ks < KST; ks++) {
    // this k-step's values at slots 16 ks + {2t, 2t+1, 2t+8, 2t+9}: aligned magnitudes
    // m = M 2^(e - E + SH) (M the 53-bit significand; with PRE oz_prep's integers, whose sign
    // bit 63 stays in hi: the digits use bytes 0..6 only) and, in sw, the word holding each
    // value's sign in bit 31
    uint32_t hi[2][4], lo[2][4], sw[2][4];
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int k = 16 * ks + 2 * t + (q & 1) + ((q >> 1) << 3);
        const double x = k < K ? Xd[(SLOT0 + k) * XST + col + 8 * r] : 0.0;
        const unsigned long long b = (unsigned long long)__double_as_longlong(x);
        sw[r][q] = (uint32_t)(b >> 32);
        unsigned long long m;
        if constexpr (PRE) m = b;
        else m = (unsigned long long)oz_align<SH>(b & 0x7FFFFFFFFFFFFFFFull, em[r]);
        hi[r][q] = (uint32_t)(m >> 32);
        lo[r][q] = (uint32_t)m;
      }
    // the fp16 pair constant of every A-fragment register (pairs (g: q0 q1), (g+8: q0 q1),
    // (g: q2 q3), (g+8: q2 q3)): 0x6400 in both halves with the low value's sign in bit 15 and
    // the high value's in bit 31 (prmt with the sign-replicating selectors 0xB and 0xF copies
    // bit 31 of each word over bytes 1 and 3)
    uint32_t v[4];
#pragma unroll
    for (int m = 0; m < 4; m++) {
      const int r = m & 1, qa = (m >> 1) * 2;
      uint32_t s2;
      asm("prmt.b32 %0, %1, %2, 0xF0B0;" : "=r"(s2) : "r"(sw[r][qa]), "r"(sw[r][qa + 1]));
      v[m] = (s2 & 0x80008000u) | 0x64006400u;
    }
#pragma unroll
    for (int j = 0; j < 7; j++) {
      // A fragment (row-major 16 x 16): rows g / g+8, slots 2t..2t+1 / 2t+8..2t+9
      const uint32_t a[4] = {oz_pair(hi[0][0], lo[0][0], hi[0][1], lo[0][1], j, v[0]),
                             oz_pair(hi[1][0], lo[1][0], hi[1][1], lo[1][1], j, v[1]),
                             oz_pair(hi[0][2], lo[0][2], hi[0][3], lo[0][3], j, v[2]),
                             oz_pair(hi[1][2], lo[1][2], hi[1][3], lo[1][3], j, v[3])};
#pragma unroll
      for (int s = 0; s + j < 7; s++) mma_f16_16816(acc[j + s], a, __ldg(bfr + (s * 2 + ks) * 32));
    }
  }
  // C fragment: acc[.][0] (row g, col 2t), [1] (g, 2t+1), [2] (g+8, 2t), [3] (g+8, 2t+1).
  // One output: the level sums lev[] of (row g + 8 r, operator row n) joined and rounded.
  auto finish = [&](const float lev[7], const int n, const int r) {
    long long l[7];
#pragma unroll
    for (int L = 0; L < 7; L++) l[L] = (long long)__float2int_rz(lev[L]);
    const long long th = l[0] * 65536LL + l[1] * 256LL + l[2];
    const long long tl = l[3] * 16777216LL + l[4] * 65536LL + l[5] * 256LL + l[6];
    const int fe = c_ozf[T][NORD][P][n];
    const int sc = em[r] + fe - 2046 - 62 + (3 - SH);
    double out;
    if (em[r] == 0x7FF) {
      out = __longlong_as_double(0x7FF8000000000000LL);
    } else if (sc >= -1022 && sc <= 900) {
      out = oz_round(th, tl, sc);
    } else if (sc < -1022) {
      out = 0.0;  // below 2^-1022: negligible against any physical value
    } else {
      const double val = fma((double)th, 4294967296.0, (double)tl);
      const int s1 = sc / 2, s2 = sc - s1;  // each <= 992: two exact power-of-two scalings
      out = (val * __longlong_as_double((long long)(s1 + 1023) << 52)) *
            __longlong_as_double((long long)(s2 + 1023) << 52);
    }
    Yd[(YROW0 + n) * XST + col + 8 * r] = out;
  };
  constexpr int RV = R - 8 * NT;  // operator rows of this n-tile that exist (1..8)
  if constexpr (RV == 6) {
    // Lanes t = 0..2 hold four outputs each (columns 2t, 2t + 1 of rows g, g + 8), lane t = 3 none:
    // lane 3 takes the (row g + 8, column 2t' + 1) output of lanes t' = 0, 1, 2 (their level sums by
    // shuffle), so every lane rounds three outputs instead of three lanes rounding four.  Same
    // values, same rounding.
    const bool hi = t == 3;
    float x[3][7];
#pragma unroll
    for (int k = 0; k < 3; k++)
#pragma unroll
      for (int L = 0; L < 7; L++) x[k][L] = __shfl_sync(0xffffffffu, acc[L][3], (lane & ~3) | k);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      float lev[7];
#pragma unroll
      for (int L = 0; L < 7; L++) lev[L] = hi ? x[k][L] : acc[L][k];
      // k = 0, 1: row g, columns 2t, 2t + 1; k = 2: row g + 8, column 2t
      const int n = 8 * NT + (hi ? 2 * k + 1 : 2 * t + (k & 1));
      finish(lev, n, hi || k == 2 ? 1 : 0);
    }
  } else if constexpr (RV <= 4) {
    // Only lanes t = 0, 1 hold outputs (columns 2t + cc < RV): lanes t = 2, 3 take the row-(g + 8)
    // outputs of lane t - 2 (their level sums by shuffle), so the rounding, the costly part, runs
    // on all four lanes of a group with half the outputs each.  Same values, same rounding.
    const bool hi = t >= 2;
    const int src = hi ? lane - 2 : lane;
    float lv[2][7];
#pragma unroll
    for (int L = 0; L < 7; L++)
#pragma unroll
      for (int cc = 0; cc < 2; cc++) {
        const float x = __shfl_sync(0xffffffffu, acc[L][2 + cc], src);
        lv[cc][L] = hi ? x : acc[L][cc];
      }
    const int tt = hi ? t - 2 : t, r = hi ? 1 : 0;
#pragma unroll
    for (int cc = 0; cc < 2; cc++) {
      const int n = 8 * NT + 2 * tt + cc;
      if (n < R) finish(lv[cc], n, r);
    }
  } else {
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int cc = 0; cc < 2; cc++) {
        const int n = 8 * NT + 2 * t + cc;
        if (n < R) {
          float lev[7];
#pragma unroll
          for (int L = 0; L < 7; L++) lev[L] = acc[L][2 * r + cc];
          finish(lev, n, r);
        }
      }
  }
}

// Parity 0: K0 staged slots from slot 0 to R0 outputs from row 0; parity 1: K1 slots from SLOT1
// to R1 outputs from YROW1.  Work units: (parity, n-tile of 8 outputs, group of 4 cells); warp w
// of nw takes units w, w + nw, ...  PRE: the operands come from oz_prep (see oz_tile).
template <int N, int T, int K0, int R0, int K1, int R1, int SLOT1, int YROW1, int NT, bool PRE, int XST>
__device__ __forceinline__ void oz_unit(const double *Xd, double *Yd, const int w, const int c0, const int lane,
                                        const int *Ems) {
  constexpr int NT0 = (R0 + 7) / 8;
  if constexpr (NT < 4) {
    if (w == NT) {
      if constexpr (NT < NT0)
        oz_tile<T, N, K0, R0, 0, 0, (K0 + 15) / 16, 0, NT, PRE, XST>(Xd, Yd, c0, lane, Ems);
      else if constexpr (NT - NT0 < (R1 + 7) / 8)
        oz_tile<T, N, K1, R1, SLOT1, YROW1, (K1 + 15) / 16, 1, NT - NT0, PRE, XST>(Xd, Yd, c0, lane, Ems);
      return;
    }
    oz_unit<N, T, K0, R0, K1, R1, SLOT1, YROW1, NT + 1, PRE, XST>(Xd, Yd, w, c0, lane, Ems);
  }
}

template <int N, int T, int K0, int R0, int K1, int R1, int SLOT1, int YROW1, bool PRE = false, int XST = 128>
__device__ __forceinline__ void oz_product(const double *Xd, double *Yd, const int warp, const int nw,
                                           const int lane, const int *Ems = nullptr) {
  constexpr int NTT = (R0 + 7) / 8 + (R1 + 7) / 8;
  static_assert(NTT <= 4, "at most 4 n-tiles");
  for (int u = warp; u < 8 * NTT; u += nw)
    oz_unit<N, T, K0, R0, K1, R1, SLOT1, YROW1, 0, PRE, XST>(Xd, Yd, u >> 3, (u & 7) * 4, lane, Ems);
}

// Sign and magnitude of an integer below 2^63 in one 64-bit word (sign in bit 63).
__device__ __forceinline__ unsigned long long oz_signmag(const long long v) {
  return v < 0 ? ((unsigned long long)(-v) | 0x8000000000000000ull) : (unsigned long long)v;
}

// The even/odd butterfly and the operand alignment of the element kernel's contraction, once per
// staged value, by the first 2 NC threads of the block (two per column of the NC: the slot pairs
// are dealt alternately, lanes l and l ^ 16 share a column).  Pairs k < NUo: slot k (x_a) and slot NUe + k
// (x_b) become x_a + x_b and x_a - x_b; the unpaired slots NUo <= k < NUe stay single.  Every
// value is aligned to the largest exponent E of its column's NK = NUe + NUo values as a 55-bit
// integer (so that sums fit 56 bits), the sums and differences are exact, and each is stored as
// sign and magnitude in its slot's 64 bits; Ems[column] = E (biased).
template <int NUe, int NUo, int XST, int NC = 128>
__device__ __forceinline__ void oz_prep(double *Xd, int *Ems, const int tid) {
  static_assert(NC % 16 == 0, "columns in groups of 16");
  if (tid >= 2 * NC) return;
  const int c = (tid & 15) | ((tid >> 5) << 4), h = (tid >> 4) & 1;
  const uint32_t *Xw = reinterpret_cast<const uint32_t *>(Xd);
  int e = 0;
#pragma unroll
  for (int k = h; k < NUe; k += 2) {
    e = max(e, (int)((Xw[2 * (k * XST + c) + 1] >> 20) & 0x7FF));
    if (k < NUo) e = max(e, (int)((Xw[2 * ((NUe + k) * XST + c) + 1] >> 20) & 0x7FF));
  }
  e = max(e, __shfl_xor_sync(0xffffffffu, e, 16));
  if (h == 0) Ems[c] = e;
#pragma unroll
  for (int k = h; k < NUe; k += 2) {
    const long long ma = oz_align<2>((unsigned long long)__double_as_longlong(Xd[k * XST + c]), e);
    if (k < NUo) {
      const long long mb = oz_align<2>((unsigned long long)__double_as_longlong(Xd[(NUe + k) * XST + c]), e);
      Xd[k * XST + c] = __longlong_as_double((long long)oz_signmag(ma + mb));
      Xd[(NUe + k) * XST + c] = __longlong_as_double((long long)oz_signmag(ma - mb));
    } else {
      Xd[k * XST + c] = __longlong_as_double((long long)oz_signmag(ma));
    }
  }
}

// Doubles per staged slot (and per output row) in the element kernel's shared memory: 32 cells x 4
// variables plus 2 doubles of padding (a slot stays 16-byte aligned for the asynchronous copies).
// A half-warp's 64-bit fragment load reads lanes g = 0..3 (consecutive doubles) of the rows 2t,
// t = 0..3, i.e. doubles 2t * XST + g: with XST = 128 all four rows start on the same bank (4-way
// conflict), with 132 rows t and t + 2 do (2-way; ~1 M conflicts per launch at N = 3), with 130
// the rows start 8 banks apart and the 16 lanes cover all 32 banks once.  Step 232.3 -> 231.2 us
// at N = 3 and 379.9 -> 377.7 us at N = 4 (runs of 40 steps; same bits).
constexpr int kElemSlot = 130;

// The element kernel's contraction: Y rows 0..NRe-1 = S_e, Y rows NRe.. = S_o, on the operands
// oz_prep made from the staged pairs (sums below slot NUe, differences from slot NUe on).  Earlier
// forms, measured on the K=32768 O-grid: the FP64 butterfly on the staged doubles with each unit
// aligning its values (steps 326 / 501 / 765 us at N = 3 / 4 / 5), and the butterfly formed in
// each unit's operands (322 us at N = 3; slower at N = 4, 5, where every n-tile redid the doubled
// alignment); oz_prep, once per value and spread over 256 threads, gives 294 / 446 / 652 us (with
// the padded slots, 308.5 / 484 / 736 us before it).
template <int N, int NUe, int NUo, int NRe, int NRo>
__device__ __forceinline__ void oz_contract(const double *Xd, double *Yd, const int warp, const int nw,
                                            const int lane, const int *Ems) {
  oz_product<N, 0, NUe, NRe, NUo, NRo, NUe, NRe, true, kElemSlot>(Xd, Yd, warp, nw, lane, Ems);
}

// The dense form: Y rows 0..NP-1 (one per node) = A (NP x NK) applied to the NK slots in their
// natural order (Fr, Fs, face points).
template <int N, int NK, int NP>
__device__ __forceinline__ void oz_contract_dense(const double *Xd, double *Yd, const int warp, const int nw,
                                                  const int lane) {
  oz_product<N, 2, NK, NP, 0, 0, NK, NP, false, kElemSlot>(Xd, Yd, warp, nw, lane);
}

// The adjoint element kernel's transposed contraction: columns 0..NUe-1 = S_e^T (even rows of the
// staged node adjoints), columns NUe.. = S_o^T (odd rows).
template <int N, int NUe, int NUo, int NRe, int NRo, int XST = 128>
__device__ __forceinline__ void oz_contract_t(const double *Xd, double *Yd, const int warp, const int nw,
                                              const int lane) {
  oz_product<N, 1, NRe, NUe, NRo, NUo, NRe, NUe, false, XST>(Xd, Yd, warp, nw, lane);
}

// ---------------------------------------------------------------- host: operator digits
// Digits and B fragments of the two parity blocks of S (even rows NRe x NUe, then odd rows
// NRo x NUo, row-major) for the tensor-core contraction.
static uint32_t oz_f16_bits(int d) {  // |d| <= 255: exact in fp16
  if (d == 0) return 0u;
  const uint32_t sign = d < 0 ? 0x8000u : 0u;
  const uint32_t m = (uint32_t)(d < 0 ? -d : d);
  int e = 0;
  while ((m >> (e + 1)) != 0u) e++;  // floor(log2 m), 0..7
  return sign | ((uint32_t)(e + 15) << 10) | ((m << (10 - e)) & 0x3FFu);
}

// Column exponents F (biased, per parity and operator row) and signed base-256 digits
// dig[p][s][k][n] (|d| <= 255) of the two parity blocks: S[n][k] = sum_s dig 256^(6-s) 2^(F-1023-55)
// up to the bits below 2^(F-1023-55) (cut).
static int oz_digits(const std::vector<double> &S, int NUe, int NUo, int NRe, int NRo, int fexp[2][kOzRows],
                     std::vector<int> &dig, std::string &err) {
  dig.assign((size_t)2 * 7 * 32 * kOzRows, 0);
  for (int p = 0; p < 2; p++) {
    const int K = p ? NUo : NUe, R = p ? NRo : NRe;
    const size_t base = p ? (size_t)NRe * NUe : 0;
    if (R > kOzRows || K > 32) { err = "tensor-core contraction: operator too large"; return -4; }
    for (int n = 0; n < kOzRows; n++) fexp[p][n] = 0;
    for (int n = 0; n < R; n++) {
      int F = 0;
      for (int k = 0; k < K; k++) {
        uint64_t b;
        std::memcpy(&b, &S[base + (size_t)n * K + k], 8);
        F = std::max(F, (int)((b >> 52) & 0x7FF));
      }
      if (F == 0x7FF) { err = "tensor-core contraction: non-finite operator entry"; return -4; }
      fexp[p][n] = F;
      for (int k = 0; k < K; k++) {
        uint64_t b;
        std::memcpy(&b, &S[base + (size_t)n * K + k], 8);
        const int e = (int)((b >> 52) & 0x7FF);
        const uint64_t M = e ? ((b & 0xFFFFFFFFFFFFFull) | (1ull << 52)) : 0;
        const int sh = e - F + 3;
        const uint64_t m = sh >= 0 ? (M << sh) : (sh > -64 ? (M >> -sh) : 0);
        const int sg = (b >> 63) ? -1 : 1;
        for (int s = 0; s < 7; s++)
          dig[(((size_t)p * 7 + s) * 32 + k) * kOzRows + n] = sg * (int)((m >> (8 * (6 - s))) & 255);
      }
    }
  }
  return 0;
}

// A: the dense rows (Np x NK, row-major) for the dense form's table (T = 2).
static int oz_upload(int N, const std::vector<double> &S, int NUe, int NUo, int NRe, int NRo,
                     const std::vector<double> &A, int Np, int NK, std::string &err) {
  if (!oz_used(N, true) && !ozd_used(N, 2)) return 0;
  static int fexp[kOzTables][2][kOzRows];
  static uint2 frag[kOzTables][2][4][7][2][32];
  std::memset(fexp, 0, sizeof(fexp));
  std::memset(frag, 0, sizeof(frag));
  for (int T = 0; T < kOzTables; T++) {
    if (T == 0 && !oz_used(N, true)) continue;
    if (T == 1 && !oz_used_t(N, true)) continue;
    if (T == 2 && !ozd_used(N, 2)) continue;
    // T = 1: the transposed blocks, S_e^T (NUe x NRe) then S_o^T (NUo x NRo)
    std::vector<double> ST;
    if (T == 1) {
      ST.resize(S.size());
      for (int r = 0; r < NRe; r++)
        for (int k = 0; k < NUe; k++) ST[(size_t)k * NRe + r] = S[(size_t)r * NUe + k];
      const size_t so = (size_t)NRe * NUe;
      for (int r = 0; r < NRo; r++)
        for (int k = 0; k < NUo; k++) ST[so + (size_t)k * NRo + r] = S[so + (size_t)r * NUo + k];
    }
    std::vector<int> dig;
    const int rc = T == 0 ? oz_digits(S, NUe, NUo, NRe, NRo, fexp[0], dig, err)
                 : T == 1 ? oz_digits(ST, NRe, NRo, NUe, NUo, fexp[1], dig, err)
                          : oz_digits(A, NK, 0, Np, 0, fexp[2], dig, err);
    if (rc) return rc;
    for (int p = 0; p < 2; p++)
      for (int nt = 0; nt < 4; nt++)
        for (int s = 0; s < 7; s++)
          for (int ks = 0; ks < 2; ks++)
            for (int lane = 0; lane < 32; lane++) {
              const int g = lane >> 2, t = lane & 3, k0 = 16 * ks + 2 * t;
              auto D = [&](int k) { return dig[(((size_t)p * 7 + s) * 32 + k) * kOzRows + 8 * nt + g]; };
              frag[T][p][nt][s][ks][lane].x = oz_f16_bits(D(k0)) | (oz_f16_bits(D(k0 + 1)) << 16);
              frag[T][p][nt][s][ks][lane].y = oz_f16_bits(D(k0 + 8)) | (oz_f16_bits(D(k0 + 9)) << 16);
            }
  }
  cudaError_t ce = cudaSuccess;
  for (int T = 0; T < kOzTables && ce == cudaSuccess; T++) {
    ce = cudaMemcpyToSymbol(c_ozf, fexp[T], sizeof(fexp[T]), ((size_t)T * 7 + N) * sizeof(fexp[T]));
    if (ce == cudaSuccess)
      ce = cudaMemcpyToSymbol(g_ozb, frag[T], sizeof(frag[T]), ((size_t)T * 7 + N) * sizeof(frag[T]));
  }
  if (ce != cudaSuccess) { err = std::string("constant upload: ") + cudaGetErrorString(ce); return -3; }
  return 0;
}
