// Geometry builder: solid mask, Bouzidi q (and dq/dr) per link, per-cell tags
// and the compacted boundary-cell records used by the fused kernels.
//
// Reference semantics:
//   world frame            geometry/primitives.py:26-53
//   hard sphere + q        geometry/primitives.py:56-174 (ray-sphere :145-172)
//   sigmoid sphere + q     geometry/smooth.py:158-248, examples/11:56-119
//   q from a mask          geometry/bouzidi.py:32-106
//   projected area         core/forces.py:199-234
#include "sim.cuh"

namespace lbm {

struct SphereSpec {
  double c[3];
  double r;
  double alpha;
  int sigmoid_mask;   // 0: dist^2 <= r^2 ; 1: sigmoid(alpha (r - dist)) > 0.5
  int bouzidi;        // 0: q = 0.5 ; 1: ray-sphere q(r)
  double disc_floor;
  double denom_eps;
};

template <class Re>
__device__ __forceinline__ void world(const Grid& g, int x, int y, int z, Re& wx, Re& wy,
                                      Re& wz) {
  const Re sx = Re(g.nx / 8.0), sy = Re(g.ny / 4.0), sz = Re(g.nz / 4.0);
  wx = (Re(x) + Re(0.5)) / sx - Re(4);
  wy = (Re(y) + Re(0.5)) / sy - Re(2);
  wz = (Re(z) + Re(0.5)) / sz - Re(2);
}

// solid code per cell: 0 fluid, 1 body
template <class Re>
__global__ void k_sphere_solid(Grid g, SphereSpec s, uint8_t* __restrict__ solid) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  const int z = idx % g.nz, t = idx / g.nz, y = t % g.ny, x = t / g.ny;
  Re wx, wy, wz;
  world<Re>(g, x, y, z, wx, wy, wz);
  const Re dx = wx - Re(s.c[0]), dy = wy - Re(s.c[1]), dz = wz - Re(s.c[2]);
  const Re r = Re(s.r);
  bool in;
  if (s.sigmoid_mask) {
    const Re d = sqrt(dx * dx + dy * dy + dz * dz);
    const Re p = Re(1) / (Re(1) + exp(-Re(s.alpha) * (r - d)));
    in = p > Re(0.5);
  } else {
    in = (dx * dx + dy * dy + dz * dz) <= Re(s.r * s.r);
  }
  solid[idx] = in ? 1 : 0;
}

__device__ __forceinline__ bool link_at(const Grid& g, const uint8_t* solid, int idx, int x,
                                        int y, int z, int j) {
  const int nx = x + ex(j), ny = y + ey(j), nz = z + ez(j);
  if (nx < 0 || nx >= g.nx || ny < 0 || ny >= g.ny || nz < 0 || nz >= g.nz) return false;
  return solid[idx] == 0 && solid[(nx * g.ny + ny) * g.nz + nz] == 1;
}

// Dense q[j][cell] (-1 where no link) and dq/dr.
template <class Re>
__global__ void k_sphere_q(Grid g, SphereSpec s, const uint8_t* __restrict__ solid,
                           Re* __restrict__ q, Re* __restrict__ dqdr) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  const int z = idx % g.nz, t = idx / g.nz, y = t % g.ny, x = t / g.ny;
  const size_t N = size_t(g.n);
  Re wx, wy, wz;
  world<Re>(g, x, y, z, wx, wy, wz);
  const Re ox = wx - Re(s.c[0]), oy = wy - Re(s.c[1]), oz = wz - Re(s.c[2]);
  const Re r = Re(s.r);
  const Re sx = Re(g.nx / 8.0), sy = Re(g.ny / 4.0), sz = Re(g.nz / 4.0);
  q[idx] = Re(-1);
  dqdr[idx] = Re(0);
#pragma unroll
  for (int j = 1; j < Q; ++j) {
    Re qv = Re(-1), dq = Re(0);
    if (link_at(g, solid, idx, x, y, z, j)) {
      if (s.bouzidi) {
        const Re rdx = Re(ex(j)) / sx, rdy = Re(ey(j)) / sy, rdz = Re(ez(j)) / sz;
        const Re a = rdx * rdx + rdy * rdy + rdz * rdz;
        const Re b = Re(2) * (ox * rdx + oy * rdy + oz * rdz);
        const Re c = ox * ox + oy * oy + oz * oz - r * r;
        const Re disc = b * b - Re(4) * a * c;
        const Re dfl = fmax(disc, Re(s.disc_floor));
        const Re sq = sqrt(dfl);
        const Re den = Re(2) * a + Re(s.denom_eps);
        const Re tt = (-b - sq) / den;
        const bool valid = (disc >= Re(0)) && (tt > Re(0)) && (tt <= Re(1));
        qv = valid ? tt : Re(0.5);
        if (valid) {
          // d t / d r through sqrt(max(disc, floor)) and clip(t, 0.01, 0.99),
          // with jax's half-cotangent rule at ties
          const Re wmax = disc > Re(s.disc_floor) ? Re(1) : (disc == Re(s.disc_floor) ? Re(0.5) : Re(0));
          dq = wmax * clip_weight<Re>(tt, Re(0.01), Re(0.99)) * (-(Re(4) * a * r) / (sq * den));
        }
        qv = fmin(fmax(qv, Re(0.01)), Re(0.99));
      } else {
        qv = Re(0.5);
      }
    }
    q[j * N + idx] = qv;
    dqdr[j * N + idx] = dq;
  }
}

// q from a solid mask (bouzidi.py:32-106): default_q on in-bounds fluid->body links.
template <class Re>
__global__ void k_q_from_solid(Grid g, const uint8_t* __restrict__ solid, Re default_q,
                               Re* __restrict__ q) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  const int z = idx % g.nz, t = idx / g.nz, y = t % g.ny, x = t / g.ny;
  const size_t N = size_t(g.n);
  q[idx] = Re(-1);
#pragma unroll
  for (int j = 1; j < Q; ++j)
    q[j * N + idx] = link_at(g, solid, idx, x, y, z, j) ? default_q : Re(-1);
}

// int32 mask (0 fluid, 1 body, 2 ground) -> solid code byte
__global__ void k_solid_from_i32(int n, const int32_t* __restrict__ m, uint8_t* __restrict__ s) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx < n) s[idx] = uint8_t(m[idx] < 0 ? 0 : (m[idx] > 2 ? 2 : m[idx]));
}

// Classify cells, assign records.  count_only: only count special cells.
template <class Re>
__global__ void k_classify(Grid g, const uint8_t* __restrict__ solid, const Re* __restrict__ q,
                           const Re* __restrict__ dqdr, uint32_t* __restrict__ tag,
                           LinkRec* __restrict__ rec, int cap, int* __restrict__ counter,
                           int count_only) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  const int z = idx % g.nz, t = idx / g.nz, y = t % g.ny, x = t / g.ny;
  const size_t N = size_t(g.n);
  uint32_t lm = 0, nbw = 0, nbl = 0;
#pragma unroll
  for (int j = 1; j < Q; ++j) {
    if (q[j * N + idx] >= Re(0)) lm |= 1u << j;
    // pull neighbour x+e_j under the streaming rules
    int px = x + ex(j), py = y + ey(j), pz = z + ez(j);
    bool ok = px >= 0 && px < g.nx;
    if (g.periodic_yz) {
      py = wrapi(py, g.ny);
      pz = wrapi(pz, g.nz);
    } else {
      ok = ok && py >= 0 && py < g.ny && pz >= 0 && pz < g.nz;
    }
    if (ok && q[opp(j) * N + (px * g.ny + py) * g.nz + pz] >= Re(0)) nbw |= 1u << j;
    const int w = ahead_wrap(g, x, y, z, ex(j), ey(j), ez(j));
    const Re qw = q[j * N + w];
    if (qw >= Re(0) && qw < Re(0.5)) nbl |= 1u << j;
  }
  const uint32_t sb = solid[idx] >= 1 ? TAG_SOLID : 0u;
  if ((lm | nbw | nbl) == 0) {
    if (!count_only) tag[idx] = sb;
    return;
  }
  const int ri = atomicAdd(counter, 1);
  if (count_only) return;
  if (ri >= cap) {
    tag[idx] = sb;
    return;
  }
  LinkRec& R = rec[ri];
  R.linkmask = lm;
  R.nb_wall = nbw;
  R.nb_low = nbl;
  R.pad = 0;
#pragma unroll
  for (int j = 0; j < Q; ++j) {
    R.q[j] = double(q[j * N + idx]);
    R.dqdr[j] = dqdr ? double(dqdr[j * N + idx]) : 0.0;
    const int w = ahead_wrap(g, x, y, z, ex(j), ey(j), ez(j));
    R.qnb[j] = (nbl >> j) & 1u ? double(q[j * N + w]) : -1.0;
  }
  tag[idx] = sb | uint32_t(ri + 1);
}

// axis-aligned box, world corners (primitives.py:177-255): solid = inside
template <class Re>
__global__ void k_box_solid(Grid g, double x0, double y0, double z0, double x1, double y1,
                            double z1, uint8_t* __restrict__ solid) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  const int z = idx % g.nz, t = idx / g.nz, y = t % g.ny, x = t / g.ny;
  Re wx, wy, wz;
  world<Re>(g, x, y, z, wx, wy, wz);
  const bool in = wx >= Re(x0) && wx <= Re(x1) && wy >= Re(y0) && wy <= Re(y1) &&
                  wz >= Re(z0) && wz <= Re(z1);
  solid[idx] = in ? 1 : 0;
}

// dense outputs of the builders for the per-op geometry functions
template <class Re>
__global__ void k_export_fields(Grid g, SphereSpec s, int with_porosity,
                                const uint8_t* __restrict__ solid, int32_t* __restrict__ solid_out,
                                Re* __restrict__ porosity) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  if (solid_out) solid_out[idx] = solid[idx];
  if (porosity && with_porosity) {
    const int z = idx % g.nz, t = idx / g.nz, y = t % g.ny, x = t / g.ny;
    Re wx, wy, wz;
    world<Re>(g, x, y, z, wx, wy, wz);
    const Re dx = wx - Re(s.c[0]), dy = wy - Re(s.c[1]), dz = wz - Re(s.c[2]);
    const Re d = sqrt(dx * dx + dy * dy + dz * dz);
    porosity[idx] = Re(1) / (Re(1) + exp(-Re(s.alpha) * (Re(s.r) - d)));
  } else if (porosity) {
    porosity[idx] = Re(solid[idx] >= 1 ? 1 : 0);
  }
}

// column flags for the projected area onto the y-z plane (body cells only)
__global__ void k_area_cols(Grid g, const uint8_t* __restrict__ solid, int* __restrict__ col) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  if (solid[idx] == 1) col[idx % (g.ny * g.nz)] = 1;
}

// Bounding box of the solid cells (any nonzero solid value): bb = {xmin,
// xmax, ymin, ymax, zmin, zmax}, initialised by the caller to empty.
__global__ void k_solid_bbox(Grid g, const uint8_t* __restrict__ solid, int* __restrict__ bb) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n || !solid[idx]) return;
  int x, y, z;
  decode(g, idx, x, y, z);
  atomicMin(bb + 0, x);
  atomicMax(bb + 1, x);
  atomicMin(bb + 2, y);
  atomicMax(bb + 3, y);
  atomicMin(bb + 4, z);
  atomicMax(bb + 5, z);
}

static inline int nblk(int n) { return (n + 255) / 256; }

template <class Re>
cudaError_t launch_sphere_fields(const Grid& g, const SphereSpec& s, uint8_t* solid, Re* q,
                                 Re* dqdr, cudaStream_t st) {
  k_sphere_solid<Re><<<nblk(g.n), 256, 0, st>>>(g, s, solid);
  k_sphere_q<Re><<<nblk(g.n), 256, 0, st>>>(g, s, solid, q, dqdr);
  return cudaGetLastError();
}

template <class Re>
cudaError_t launch_q_from_solid(const Grid& g, const uint8_t* solid, double dq, Re* q,
                                cudaStream_t st) {
  k_q_from_solid<Re><<<nblk(g.n), 256, 0, st>>>(g, solid, Re(dq), q);
  return cudaGetLastError();
}

cudaError_t launch_solid_from_i32(int n, const int32_t* m, uint8_t* s, cudaStream_t st) {
  k_solid_from_i32<<<nblk(n), 256, 0, st>>>(n, m, s);
  return cudaGetLastError();
}

template <class Re>
cudaError_t launch_classify(const Grid& g, const uint8_t* solid, const Re* q, const Re* dqdr,
                            uint32_t* tag, LinkRec* rec, int cap, int* counter, int count_only,
                            cudaStream_t st) {
  k_classify<Re><<<nblk(g.n), 256, 0, st>>>(g, solid, q, dqdr, tag, rec, cap, counter,
                                            count_only);
  return cudaGetLastError();
}

template <class Re>
cudaError_t launch_box_fields(const Grid& g, const double lo[3], const double hi[3],
                              uint8_t* solid, Re* q, cudaStream_t st) {
  k_box_solid<Re><<<nblk(g.n), 256, 0, st>>>(g, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], solid);
  k_q_from_solid<Re><<<nblk(g.n), 256, 0, st>>>(g, solid, Re(0.5), q);
  return cudaGetLastError();
}

template <class Re>
cudaError_t launch_export_fields(const Grid& g, const SphereSpec& s, int with_porosity,
                                 const uint8_t* solid, int32_t* solid_out, Re* porosity,
                                 cudaStream_t st) {
  k_export_fields<Re><<<nblk(g.n), 256, 0, st>>>(g, s, with_porosity, solid, solid_out, porosity);
  return cudaGetLastError();
}

cudaError_t launch_solid_bbox(const Grid& g, const uint8_t* solid, int* bb, cudaStream_t st) {
  k_solid_bbox<<<nblk(g.n), 256, 0, st>>>(g, solid, bb);
  return cudaGetLastError();
}

cudaError_t launch_area_cols(const Grid& g, const uint8_t* solid, int* col, cudaStream_t st) {
  k_area_cols<<<nblk(g.n), 256, 0, st>>>(g, solid, col);
  return cudaGetLastError();
}

// Per-cell porosity and dp/dr of a sigmoid sphere (sphere_porosity), once per
// geometry: the step and adjoint kernels read them instead of evaluating the
// sigmoid (three divisions, a square root and an exponential) every step.
template <class Re>
__global__ void k_sphere_porosity(Grid g, SphereP<Re> sp, Re* __restrict__ p,
                                  Re* __restrict__ dpdr) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= g.n) return;
  int x, y, z;
  decode(g, idx, x, y, z);
  Re d;
  p[idx] = sphere_porosity<Re>(sp, x, y, z, &d);
  dpdr[idx] = d;
}

template <class Re>
cudaError_t launch_sphere_porosity(const Grid& g, const SphereP<Re>& sp, Re* p, Re* dpdr,
                                   cudaStream_t st) {
  k_sphere_porosity<Re><<<(g.n + 255) / 256, 256, 0, st>>>(g, sp, p, dpdr);
  return cudaGetLastError();
}

template cudaError_t launch_sphere_porosity<float>(const Grid&, const SphereP<float>&, float*,
                                                   float*, cudaStream_t);
template cudaError_t launch_sphere_porosity<double>(const Grid&, const SphereP<double>&, double*,
                                                    double*, cudaStream_t);
template cudaError_t launch_sphere_fields<float>(const Grid&, const SphereSpec&, uint8_t*, float*,
                                                 float*, cudaStream_t);
template cudaError_t launch_sphere_fields<double>(const Grid&, const SphereSpec&, uint8_t*,
                                                  double*, double*, cudaStream_t);
template cudaError_t launch_q_from_solid<float>(const Grid&, const uint8_t*, double, float*,
                                                cudaStream_t);
template cudaError_t launch_q_from_solid<double>(const Grid&, const uint8_t*, double, double*,
                                                 cudaStream_t);
template cudaError_t launch_box_fields<float>(const Grid&, const double*, const double*,
                                              uint8_t*, float*, cudaStream_t);
template cudaError_t launch_box_fields<double>(const Grid&, const double*, const double*,
                                               uint8_t*, double*, cudaStream_t);
template cudaError_t launch_export_fields<float>(const Grid&, const SphereSpec&, int,
                                                 const uint8_t*, int32_t*, float*, cudaStream_t);
template cudaError_t launch_export_fields<double>(const Grid&, const SphereSpec&, int,
                                                  const uint8_t*, int32_t*, double*, cudaStream_t);
template cudaError_t launch_classify<float>(const Grid&, const uint8_t*, const float*,
                                            const float*, uint32_t*, LinkRec*, int, int*, int,
                                            cudaStream_t);
template cudaError_t launch_classify<double>(const Grid&, const uint8_t*, const double*,
                                             const double*, uint32_t*, LinkRec*, int, int*, int,
                                             cudaStream_t);

}  // namespace lbm
