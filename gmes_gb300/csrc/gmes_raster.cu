// Material-map builder: rasterise the geometry list into a component's u8
// class map on the GPU.  Compiled with --fmad=false: the inclusion tests must
// round exactly as the reference's FP64 geometry code (and this package's
// numpy restatement of it) so that points on a shape's surface fall on the
// same side.
#include <cmath>

#include "gmes_internal.cuh"

namespace gmes {
namespace {

// Yee coordinate of index n along `axis` (gmes/geometry.py:360-732).
__device__ __forceinline__ double coord(const GridDev& g, const double* half, int c, int axis,
                                        int64_t n) {
  return ((double)n + yee_offset(c, axis)) * g.dr[axis] - half[axis];
}

__device__ bool inside(const gmes_shape& s, double x, double y, double z) {
  if (s.type == GMES_SHAPE_ALL) return true;
  if (x < s.lo[0] || x > s.hi[0] || y < s.lo[1] || y > s.hi[1] || z < s.lo[2] || z > s.hi[2])
    return false;
  const double rx = x - s.center[0], ry = y - s.center[1], rz = z - s.center[2];
  switch (s.type) {
    case GMES_SHAPE_SPHERE:  // src/pygeom.pyx:962-970
      return sqrt(rx * rx + ry * ry + rz * rz) <= s.p[0];
    case GMES_SHAPE_BLOCK: {  // src/pygeom.pyx:808-818
      for (int a = 0; a < 3; ++a) {
        const double pr = s.m[3 * a] * rx + s.m[3 * a + 1] * ry + s.m[3 * a + 2] * rz;
        if (!(fabs(pr) <= s.p[a])) return false;
      }
      return true;
    }
    case GMES_SHAPE_ELLIPSOID: {  // src/pygeom.pyx:877-887
      double q[3];
      for (int a = 0; a < 3; ++a)
        q[a] = (s.m[3 * a] * rx + s.m[3 * a + 1] * ry + s.m[3 * a + 2] * rz) * s.p[a];
      return q[0] * q[0] + q[1] * q[1] + q[2] * q[2] <= 1.0;
    }
    case GMES_SHAPE_CONE: {  // src/pygeom.pyx:633-652
      const double proj = s.axis[0] * rx + s.axis[1] * ry + s.axis[2] * rz;
      if (!(fabs(proj) <= 0.5 * s.p[2])) return false;
      if (s.p[1] == s.p[0] && isinf(s.p[0])) return true;
      const double radius = s.p[0] + (proj / s.p[2] + 0.5) * (s.p[1] - s.p[0]);
      const double px = rx - proj * s.axis[0], py = ry - proj * s.axis[1],
                   pz = rz - proj * s.axis[2];
      return sqrt(px * px + py * py + pz * pz) <= fabs(radius);
    }
    case GMES_SHAPE_SHELL: {  // src/pygeom.pyx:1127-1132
      for (int b = 0; b < s.nbox && b < 6; ++b)
        if (s.box_lo[b][0] <= x && x <= s.box_hi[b][0] && s.box_lo[b][1] <= y &&
            y <= s.box_hi[b][1] && s.box_lo[b][2] <= z && z <= s.box_hi[b][2])
          return true;
      return false;
    }
    default:
      return false;
  }
}

__global__ void k_raster(const GridDev g, int c, const gmes_shape* shapes, int nshapes,
                         const uint8_t* lut, double h0, double h1, double h2) {
  const int64_t np = g.npts[c];
  const double half[3] = {h0, h1, h2};
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < np;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / g.st[c][0];
    const int64_t rem = t - i * g.st[c][0];
    const int64_t j = rem / g.st[c][1];
    const int64_t k = rem - j * g.st[c][1];
    const int own = c % 3, a1 = (own + 1) % 3, a2 = (own + 2) % 3;
    const int64_t x[3] = {i, j, k};
    uint8_t id = 0;
    // ghost planes (gmes/fdtd.py:365-470): E last plane / H first plane
    // along the two non-own axes are Dummy
    const bool ghost = c < 3 ? (x[a1] == g.sh[c][a1] - 1 || x[a2] == g.sh[c][a2] - 1)
                             : (x[a1] == 0 || x[a2] == 0);
    if (!ghost) {
      const double px = coord(g, half, c, 0, i), py = coord(g, half, c, 1, j),
                   pz = coord(g, half, c, 2, k);
      int owner = 0;
      for (int q = nshapes - 1; q > 0; --q)
        if (inside(shapes[q], px, py, pz)) {
          owner = q;
          break;
        }
      int under = -1;
      if (shapes[owner].compound && owner > 0) {
        under = 0;
        for (int q = owner - 1; q > 0; --q)
          if (inside(shapes[q], px, py, pz)) {
            under = q;
            break;
          }
      }
      id = lut[(int64_t)owner * (nshapes + 1) + under + 1];
    }
    const_cast<uint8_t*>(g.cls[c])[t] = id;
  }
}

}  // namespace

cudaError_t launch_raster(const gmes_grid_desc& gd, const GridDev& d, int c,
                          const gmes_shape* shapes, int nshapes, const uint8_t* lut,
                          cudaStream_t s) {
  const int64_t np = d.npts[c];
  const int blocks = (int)((np + 255) / 256 < 152 * 64 ? (np + 255) / 256 : 152 * 64);
  k_raster<<<blocks, 256, 0, s>>>(d, c, shapes, nshapes, lut, gd.half[0], gd.half[1],
                                  gd.half[2]);
  return cudaGetLastError();
}

}  // namespace gmes
