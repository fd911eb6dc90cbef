// Shared device-side structures of the fused solver: grid, boundary-cell
// records, kernel argument blocks and the pull / Bouzidi / Zou-He helpers.
//
// Data layout in HBM (identical to jax_lbm's arrays, state.py:41-44):
//   populations  [19][nx][ny][nz]  z fastest (structure of arrays)
//   tag          [nx][ny][nz] uint32: bit 31 = hard-solid cell, bits 0..30 =
//                1 + index of the cell's LinkRec (0 = plain cell)
//   LinkRec[]    one record per "special" cell: a cell that owns a Bouzidi
//                link, is the target of one, or is the second fluid cell of a
//                q < 0.5 link.  Only these cells read anything beyond the pull.
#pragma once

#include "lbm_core.cuh"

namespace lbm {

constexpr uint32_t TAG_SOLID = 0x80000000u;
constexpr uint32_t TAG_INDEX = 0x7FFFFFFFu;

struct alignas(16) LinkRec {
  uint32_t linkmask;  // bit j: q[j](x) >= 0  (direction j from x hits a wall)
  uint32_t nb_wall;   // bit j: pull neighbour x+e_j has q[opp j] >= 0
  uint32_t nb_low;    // bit j: 0 <= q[j](wrap(x+e_j)) < 0.5
  uint32_t pad;
  double q[Q];        // q[j](x)
  double qnb[Q];      // q[j](wrap(x+e_j)) for nb_low bits
  double dqdr[Q];     // d q[j](x) / d r
};

// Unsigned division by a runtime constant with a multiply-high
// (Granlund-Montgomery): q = (umulhi(n, mul) + n) >> shift, exact for n < 2^31.
struct FastDiv {
  uint32_t d, mul, shift;
  __host__ __device__ __forceinline__ uint32_t div(uint32_t n) const {
#ifdef __CUDA_ARCH__
    return (__umulhi(n, mul) + n) >> shift;
#else
    return uint32_t(((uint64_t(n) * mul >> 32) + n) >> shift);
#endif
  }
};
inline FastDiv make_fastdiv(uint32_t d) {
  FastDiv f;
  f.d = d;
  uint32_t l = 0;
  while ((1ull << l) < d) ++l;
  f.shift = l;
  f.mul = uint32_t(((1ull << 32) * ((1ull << l) - d)) / d + 1);
  return f;
}

struct Grid {
  int nx, ny, nz;
  int n;              // nx*ny*nz
  int periodic_yz;
  FastDiv dz, dy;     // divide by nz, by ny
};

inline Grid make_grid(int nx, int ny, int nz, int periodic) {
  Grid g;
  g.nx = nx;
  g.ny = ny;
  g.nz = nz;
  g.n = nx * ny * nz;
  g.periodic_yz = periodic ? 1 : 0;
  g.dz = make_fastdiv(uint32_t(nz));
  g.dy = make_fastdiv(uint32_t(ny));
  return g;
}

__device__ __forceinline__ void decode(const Grid& g, int idx, int& x, int& y, int& z) {
  const uint32_t t = g.dz.div(uint32_t(idx));
  z = idx - int(t) * g.nz;
  const uint32_t xx = g.dy.div(t);
  y = int(t) - int(xx) * g.ny;
  x = int(xx);
}

// flags of StepArgs::flags
enum : int {
  SF_SMAG = 1 << 0,
  SF_SOLID_HARD = 1 << 1,
  SF_SOLID_SPHERE = 1 << 2,   // analytic sigmoid porosity
  SF_SOLID_FIELD = 1 << 3,    // porosity array
  SF_GUARD_PRE = 1 << 4,
  SF_GUARD_POST = 1 << 5,
  SF_FORCE = 1 << 6,
  SF_COLLIDE_ONLY = 1 << 7,   // input is the reference-layout f (no pull)
  SF_STREAM_ONLY = 1 << 8,    // output is the reference-layout post-BC f
  SF_INLET_FACE = 1 << 9,     // per-(y,z) inlet velocity
  SF_NO_INLET = 1 << 10,
  SF_NO_OUTLET = 1 << 11,
  SF_EMIT_F = 1 << 12,        // also write the post-BC f (after the post guard) to f_emit
};

template <class Re> struct SphereP {
  Re c[3];
  Re r;
  Re alpha;
  Re sx, sy, sz;   // cells per world unit: nx/8, ny/4, nz/4
};

template <class Re> struct StepArgs {
  const void* src;        // populations S_{k-1} (storage type) or f_0 (Re)
  void* dst;              // populations S_k (storage type) or post-BC f (Re)
  const uint32_t* tag;
  const LinkRec* rec;
  Grid g;
  Consts<Re> K;
  Re tau;
  Re c18cs2;              // 18 Cs^2
  int flags;
  Re u_in[3];
  const Re* u_face;       // [3][ny][nz]
  Re rho_out;
  SphereP<Re> sph;
  const Re* porosity;     // [n] porosity field (also filled for a sigmoid sphere)
  const Re* dpdr;         // [n] dp/dr of a sigmoid sphere, else null
  Re guard_reset[Q];
  // 16-bit storage holds f_i minus an offset: the rest equilibrium w_i inside
  // the box `near` around the body (where u ~ 0), the free-stream equilibrium
  // f_eq(1, (u_in, 0, 0)) elsewhere -- so every cell stores a small deviation
  Re soff[Q];             // outside the box
  Re soff_near[Q];        // inside the box
  int near[6];            // [x0, x1) x [y0, y1) x [z0, z1); empty when x0 >= x1
  const int* spec_pairs;  // pairs the pair kernels run on their per-cell path (nz even)
  int spec_count;
  double* force_partials; // [gridDim.x][3]
  unsigned long long* guard_count;
  void* f_emit;           // SF_EMIT_F: the post-BC f of the pull (Re), [19][n]
};

__device__ __forceinline__ int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

struct Near {
  int b[6];
};

// ---- storage offsets of 16-bit populations ----------------------------------
__device__ __forceinline__ bool in_near(const int b[6], int x, int y, int z) {
  return x >= b[0] && x < b[1] && y >= b[2] && y < b[3] && z >= b[4] && z < b[5];
}

// In-box masks of a cell's neighbourhood, one bit per offset along each
// axis: bit k of mx is "x + k - 1 inside the box" (x never wraps), of my
// likewise with y wrapped, and of mz for z - 1 .. z + zc (wrapped), zc = 1
// (one cell) or 2 (a z-pair).  The source x - e_i of direction i is inside
// iff bit 1 - e_x of mx, 1 - e_y of my and 1 - e_z of mz are all set.
struct NearMask {
  unsigned mx, my, mz;
  __device__ __forceinline__ NearMask(const Grid& g, const int b[6], int x, int y, int z, int zc) {
    auto in = [](int v, int lo, int hi) { return unsigned(v >= lo && v < hi); };
    mx = in(x - 1, b[0], b[1]) | (in(x, b[0], b[1]) << 1) | (in(x + 1, b[0], b[1]) << 2);
    my = in(wrapi(y - 1, g.ny), b[2], b[3]) | (in(y, b[2], b[3]) << 1) |
         (in(wrapi(y + 1, g.ny), b[2], b[3]) << 2);
    mz = in(wrapi(z - 1, g.nz), b[4], b[5]) | (in(z, b[4], b[5]) << 1) |
         (in(wrapi(z + 1, g.nz), b[4], b[5]) << 2);
    if (zc == 2) mz |= in(wrapi(z + 2, g.nz), b[4], b[5]) << 3;
  }
  // 0: the whole neighbourhood outside, 1: inside, 2: mixed
  __device__ __forceinline__ int cls(int zc) const {
    const unsigned full_z = zc == 2 ? 15u : 7u;
    if (mx == 0u || my == 0u || mz == 0u) return 0;
    if (mx == 7u && my == 7u && mz == full_z) return 1;
    return 2;
  }
  // class of the pull source x - e_i of the cell at z (lane 0)
  __device__ __forceinline__ bool src_in(int i) const {
    return ((mx >> (1 - ex(i))) & (my >> (1 - ey(i))) & (mz >> (1 - ez(i))) & 1u) != 0u;
  }
  // class of the neighbour x + e_i of the cell at z (lane 0)
  __device__ __forceinline__ bool nbr_in(int i) const {
    return ((mx >> (1 + ex(i))) & (my >> (1 + ey(i))) & (mz >> (1 + ez(i))) & 1u) != 0u;
  }
  __device__ __forceinline__ bool self_in() const { return ((mx & my & mz) >> 1) & 1u; }
};

__device__ __forceinline__ int near_class(const Grid& g, const int b[6], int x, int y, int z,
                                          int zc) {
  // x never wraps: most cells are decided by x alone
  if (x + 1 < b[0] || x - 1 >= b[1]) return 0;
  return NearMask(g, b, x, y, z, zc).cls(zc);
}

// A z-pair (z even) that the packed pair kernels run on their per-cell path:
// a boundary record on either cell, an x face (fallback pull and Zou-He), a
// non-periodic y/z edge, or (when the storage offsets matter, use_class) a
// neighbourhood that straddles the body box.  The pair kernels' interior
// blocks skip these pairs; their list blocks compute them from the list built
// with this same predicate.  (Listing the x faces rather than testing for
// them in the interior measured 94 us against 100 us per 16-bit step at
// 256x128x128.)
__device__ __forceinline__ bool pair_special(const Grid& g, const int near[6], bool use_class,
                                             int x, int y, int z, uint32_t t0, uint32_t t1) {
  const bool xface = x == 0 || x == g.nx - 1;
  bool sp = ((t0 | t1) & TAG_INDEX) || xface;
  if (!g.periodic_yz) sp = sp || y == 0 || y == g.ny - 1 || z == 0 || z + 2 == g.nz;
  if (use_class && !sp) sp = near_class(g, near, x, y, z, 2) == 2;
  return sp;
}

template <class Re>
__device__ __forceinline__ Re soff_at(const StepArgs<Re>& a, int x, int y, int z, int i) {
  return in_near(a.near, x, y, z) ? a.soff_near[i] : a.soff[i];
}

// Pull source of direction i for cell (x,y,z) following streaming.py:109-142:
// x is never periodic, y/z are periodic or clamped; any out-of-range axis
// makes the cell keep its own value.
__device__ __forceinline__ int pull_src(int i, const Grid& g, int idx, int x, int y, int z) {
  int sx = x - ex(i), sy = y - ey(i), sz = z - ez(i);
  bool fb = false;
  if (ex(i) != 0) fb |= (sx < 0) | (sx >= g.nx);
  if (ey(i) != 0) {
    if (g.periodic_yz) sy = wrapi(sy, g.ny); else fb |= (sy < 0) | (sy >= g.ny);
  }
  if (ez(i) != 0) {
    if (g.periodic_yz) sz = wrapi(sz, g.nz); else fb |= (sz < 0) | (sz >= g.nz);
  }
  return fb ? idx : ((sx * g.ny + sy) * g.nz + sz);
}

// Cell x + e_i wrapped in all three axes (jnp.roll semantics, streaming.py:166-172).
__device__ __forceinline__ int ahead_wrap(const Grid& g, int x, int y, int z, int dx, int dy,
                                          int dz) {
  return (wrapi(x + dx, g.nx) * g.ny + wrapi(y + dy, g.ny)) * g.nz + wrapi(z + dz, g.nz);
}

// Zou-He velocity inlet at x = 0 (boundary.py:35-124).
template <class Re>
__device__ __forceinline__ void zou_he_inlet(Re f[Q], Re ux, Re uy, Re uz) {
  const Re k0 = f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18];
  const Re kn = f[2] + f[8] + f[10] + f[12] + f[14];
  const Re rho = (k0 + Re(2) * kn) / (Re(1) - ux);
  const Re c3 = Re(1.0 / 3.0) * rho, c6 = Re(1.0 / 6.0) * rho;
  f[1] = f[2] + c3 * ux;
  f[7] = f[10] + c6 * (ux + uy);
  f[9] = f[8] + c6 * (ux - uy);
  f[11] = f[14] + c6 * (ux + uz);
  f[13] = f[12] + c6 * (ux - uz);
}

// Zou-He pressure outlet at x = nx-1 with u_y = u_z = 0 (boundary.py:127-200).
template <class Re>
__device__ __forceinline__ void zou_he_outlet(Re f[Q], Re rho_out) {
  const Re k0 = f[0] + f[3] + f[4] + f[5] + f[6] + f[15] + f[16] + f[17] + f[18];
  const Re kp = f[1] + f[7] + f[9] + f[11] + f[13];
  const Re ux = Re(-1) + (k0 + Re(2) * kp) / rho_out;
  const Re c3 = Re(1.0 / 3.0) * rho_out * ux, c6 = Re(1.0 / 6.0) * rho_out * ux;
  f[2] = f[1] - c3;
  f[10] = f[7] - c6;
  f[8] = f[9] - c6;
  f[14] = f[11] - c6;
  f[12] = f[13] - c6;
}

// Sigmoid porosity of the analytic sphere at cell (x,y,z), smooth.py:34-115:
// p = sigmoid(alpha (r - |x_world - c|)).
template <class Re>
__device__ __forceinline__ Re sphere_porosity(const SphereP<Re>& s, int x, int y, int z,
                                              Re* dpdr) {
  const Re wx = (Re(x) + Re(0.5)) / s.sx - Re(4);
  const Re wy = (Re(y) + Re(0.5)) / s.sy - Re(2);
  const Re wz = (Re(z) + Re(0.5)) / s.sz - Re(2);
  const Re dx = wx - s.c[0], dy = wy - s.c[1], dz = wz - s.c[2];
  const Re d = sqrt(dx * dx + dy * dy + dz * dz);
  const Re p = Re(1) / (Re(1) + exp(-s.alpha * (s.r - d)));
  if (dpdr) *dpdr = s.alpha * p * (Re(1) - p);
  return p;
}

// Guard test of state.py:161-166 / examples/10:164-167 on (rho, j):
// rho < 0.3, rho > 2, |u| > 0.4 (tested as |j|^2 > 0.16 rho^2, rho being in
// [0.3, 2] by then), or rho NaN (the first comparison fails for NaN).
template <class Re>
__device__ __forceinline__ bool unstable_rj(Re rho, Re jx, Re jy, Re jz) {
  const Re j2 = jx * jx + jy * jy + jz * jz;
  return !(rho >= Re(0.3) && rho <= Re(2.0)) || (j2 > Re(0.16) * rho * rho);
}

// Pull offsets of one cell, hoisted out of the 19-direction loop: source
// coordinate s = x - e along each axis, with validity (x never periodic;
// y/z periodic or clamped, streaming.py:109-142).
struct PullIdx {
  int xo[3], yo[3], zo[3];   // index 0: e = -1, 1: e = 0, 2: e = +1
  bool xv[3], yv[3], zv[3];
  __device__ __forceinline__ PullIdx(const Grid& g, int x, int y, int z) {
    const int nyz = g.ny * g.nz;
    xo[0] = (x + 1) * nyz; xo[1] = x * nyz; xo[2] = (x - 1) * nyz;
    xv[0] = x < g.nx - 1; xv[1] = true; xv[2] = x > 0;
    int yp = y + 1, ym = y - 1, zp = z + 1, zm = z - 1;
    if (g.periodic_yz) {
      yp = yp >= g.ny ? yp - g.ny : yp;
      ym = ym < 0 ? ym + g.ny : ym;
      zp = zp >= g.nz ? zp - g.nz : zp;
      zm = zm < 0 ? zm + g.nz : zm;
      yv[0] = yv[2] = zv[0] = zv[2] = true;
    } else {
      yv[0] = y < g.ny - 1; yv[2] = y > 0;
      zv[0] = z < g.nz - 1; zv[2] = z > 0;
    }
    yv[1] = zv[1] = true;
    yo[0] = yp * g.nz; yo[1] = y * g.nz; yo[2] = ym * g.nz;
    zo[0] = zp; zo[1] = z; zo[2] = zm;
  }
  __device__ __forceinline__ int src(int i, int idx) const {
    const int a = 1 + ex(i), b = 1 + ey(i), c = 1 + ez(i);
    const bool ok = xv[a] && yv[b] && zv[c];
    return ok ? xo[a] + yo[b] + zo[c] : idx;
  }
  // forward pull of direction i reads (x - e_i) (no fallback)
  __device__ __forceinline__ bool valid(int i) const {
    return xv[1 + ex(i)] && yv[1 + ey(i)] && zv[1 + ez(i)];
  }
  __device__ __forceinline__ int raw(int i) const {
    return xo[1 + ex(i)] + yo[1 + ey(i)] + zo[1 + ez(i)];
  }
};

// Neighbour offsets of a cell away from the domain faces: cell x + d (each
// component d in {-1,0,1}) is idx + ox[d+1] + oy[d+1] + oz[d+1], with the
// periodic y/z wrap folded in.  `face` marks cells where some neighbour is
// out of range (x = 0 / nx-1 always; y/z edges when not periodic); those use
// PullIdx and its fallback rule.
struct NbrOff {
  int ox[3], oy[3], oz[3];
  bool face;
  __device__ __forceinline__ NbrOff(const Grid& g, int x, int y, int z) {
    const int nyz = g.ny * g.nz;
    ox[0] = -nyz; ox[1] = 0; ox[2] = nyz;
    oy[0] = -g.nz + (y == 0 ? nyz : 0);
    oy[1] = 0;
    oy[2] = g.nz - (y == g.ny - 1 ? nyz : 0);
    oz[0] = -1 + (z == 0 ? g.nz : 0);
    oz[1] = 0;
    oz[2] = 1 - (z == g.nz - 1 ? g.nz : 0);
    face = (x == 0) || (x == g.nx - 1);
    if (!g.periodic_yz) face = face || y == 0 || y == g.ny - 1 || z == 0 || z == g.nz - 1;
  }
  // source of the pull of direction i: x - e_i
  __device__ __forceinline__ int pull(int i, int idx) const {
    return idx + ox[1 - ex(i)] + oy[1 - ey(i)] + oz[1 - ez(i)];
  }
  // x + e_j
  __device__ __forceinline__ int push(int j, int idx) const {
    return idx + ox[1 + ex(j)] + oy[1 + ey(j)] + oz[1 + ez(j)];
  }
};

// Post-stream, post-boundary populations f_k of cell (x,y,z) from the stored
// post-collision populations S_{k-1}: pull (streaming.py:109-142), Bouzidi on
// the cell's wall links (streaming.py:148-183), Zou-He inlet/outlet
// (boundary.py:35-200).
// `tab` (optional): per-direction pull bases src + i N - (e_x nyz + e_y nz +
// e_z) from the launch's argument block, so an interior pull address is one
// table entry plus the cell index and its y / z wrap corrections.
template <class St>
__device__ __forceinline__ void pull_post_bc(const StepArgs<typename Storage<St>::Re>& a,
                                             const St* __restrict__ src, int idx, int x, int y,
                                             int z, uint32_t tag,
                                             typename Storage<St>::Re f[Q],
                                             const St* const* tab = nullptr) {
  using Re = typename Storage<St>::Re;
  using S = Storage<St>;
  const Grid& g = a.g;
  const size_t N = size_t(g.n);
  const NbrOff O(g, x, y, z);
  // offset classes matter only for 16-bit storage (FP32/FP64 store f itself)
  constexpr bool offs = sizeof(St) == 2;
  const NearMask M(g, a.near, x, y, z, 1);
  const int cls = offs ? M.cls(1) : 0;
  if (!O.face && cls != 2 && tab) {
    const int nyz = g.ny * g.nz;
    const int wym = y == 0 ? nyz : 0;             // e_y = +1 pulls y - 1
    const int wyp = y == g.ny - 1 ? -nyz : 0;     // e_y = -1 pulls y + 1
    const int wzm = z == 0 ? g.nz : 0;            // e_z = +1 pulls z - 1
    const int wzp = z == g.nz - 1 ? -g.nz : 0;    // e_z = -1 pulls z + 1
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      const int b = idx + (ey(i) == 1 ? wym : (ey(i) == -1 ? wyp : 0)) +
                    (ez(i) == 1 ? wzm : (ez(i) == -1 ? wzp : 0));
      f[i] = S::ld(tab[i] + b, cls ? a.soff_near[i] : a.soff[i]);
    }
  } else if (!O.face && cls != 2) {
#pragma unroll
    for (int i = 0; i < Q; ++i)
      f[i] = S::ld(src + i * N + O.pull(i, idx), cls ? a.soff_near[i] : a.soff[i]);
  } else {
    const PullIdx P(g, x, y, z);
#pragma unroll
    for (int i = 0; i < Q; ++i) {
      // offset class of the source cell (the cell itself on the fallback)
      const bool in = P.valid(i) ? M.src_in(i) : M.self_in();
      f[i] = S::ld(src + i * N + P.src(i, idx), in ? a.soff_near[i] : a.soff[i]);
    }
  }
  const uint32_t ri = tag & TAG_INDEX;
  if (ri) {
    const LinkRec& r = a.rec[ri - 1];
    const uint32_t lm = r.linkmask;
    const bool own_near = M.self_in();
#pragma unroll
    for (int i = 1; i < Q; ++i) {
      const int io = opp(i);
      if (lm & (1u << io)) {
        const Re qv = Re(r.q[io]);
        const Re s_opp = S::ld(src + io * N + idx, own_near ? a.soff_near[io] : a.soff[io]);
        if (qv >= Re(0.5)) {
          const Re s_i = S::ld(src + i * N + idx, own_near ? a.soff_near[i] : a.soff[i]);
          const Re inv2q = Re(1) / (Re(2) * fmin(qv, Re(1)));
          f[i] = inv2q * s_opp + (Re(1) - inv2q) * s_i;
        } else {
          const int nb = ahead_wrap(g, x, y, z, ex(i), ey(i), ez(i));
          const Re s_nb = S::ld(src + io * N + nb, M.nbr_in(i) ? a.soff_near[io] : a.soff[io]);
          const Re twoq = Re(2) * fmax(qv, Re(0));
          f[i] = twoq * s_opp + (Re(1) - twoq) * s_nb;
        }
      }
    }
  }
  if (x == 0 && !(a.flags & SF_NO_INLET)) {
    Re ux = a.u_in[0], uy = a.u_in[1], uz = a.u_in[2];
    if (a.flags & SF_INLET_FACE) {
      const int fi = y * g.nz + z, fn = g.ny * g.nz;
      ux = a.u_face[fi];
      uy = a.u_face[fn + fi];
      uz = a.u_face[2 * fn + fi];
    }
    zou_he_inlet<Re>(f, ux, uy, uz);
  }
  if (x == g.nx - 1 && !(a.flags & SF_NO_OUTLET)) zou_he_outlet<Re>(f, a.rho_out);
}

// Block-wide sum of three doubles; thread 0 writes them to out[slot*3].
__device__ __forceinline__ void block_sum3_store_at(double a, double b, double c, double* out,
                                                    int slot) {
  __shared__ double sh[3][32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
    c += __shfl_down_sync(0xffffffffu, c, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) { sh[0][wid] = a; sh[1][wid] = b; sh[2][wid] = c; }
  __syncthreads();
  if (wid == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    a = lane < nw ? sh[0][lane] : 0.0;
    b = lane < nw ? sh[1][lane] : 0.0;
    c = lane < nw ? sh[2][lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_down_sync(0xffffffffu, a, o);
      b += __shfl_down_sync(0xffffffffu, b, o);
      c += __shfl_down_sync(0xffffffffu, c, o);
    }
    if (lane == 0) {
      out[3 * slot + 0] = a;
      out[3 * slot + 1] = b;
      out[3 * slot + 2] = c;
    }
  }
}

__device__ __forceinline__ void block_sum3_store(double a, double b, double c, double* out) {
  block_sum3_store_at(a, b, c, out, blockIdx.x);
}

}  // namespace lbm
