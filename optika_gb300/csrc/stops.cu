// The stop solver's Newton iterations on the device.
//
// optika/systems/_sequential.py:396-693 (_calc_rayfunction_stops_only)
// finds, for each pair of a point on the first stop's boundary and one on
// the last stop's, the free component of the ray at the first stop (its
// direction, or its position when that stop's aperture is angular) that
// lands the ray on the target point, by Newton's method with a
// forward-difference Jacobian.  Here one thread solves one pair (at one
// wavelength): every iteration traces the ray and its two perturbations
// through the surfaces between the stops with the trace's device functions,
// expresses the result in the last stop's frame in float64 and applies the
// 2 x 2 update in float64, with no host round trip per iteration.
#include "trace_kernel.cuh"

namespace otx {

struct StopArgs {
  otx_stop_solve s;
  otx_surface first;  // the first stop's sag (for a free position on it)
};

// Residual of the ray whose free component is (x, y): target minus the
// ray's point (or direction) in the last stop's frame.
__device__ void stop_residual(const otx_system& sys, const StopArgs& A, int64_t i, double x,
                              double y, double& fx, double& fy) {
  const otx_stop_solve& s = A.s;
  const int64_t n = s.count;
  const double* P = reinterpret_cast<const double*>(s.position);
  const double* D = reinterpret_cast<const double*>(s.direction);
  double p[3] = {P[i], P[n + i], P[2 * n + i]};
  double d[3] = {D[i], D[n + i], D[2 * n + i]};
  if (s.free_position) {
    float gx, gy;
    p[0] = x;
    p[1] = y;
    p[2] = (double)sag_eval(A.first.sag_type, A.first, (float)x, (float)y, gx, gy);
  } else {
    d[0] = x;
    d[1] = y;
    d[2] = sqrt(1.0 - (x * x + y * y));
  }
  Ray r;
  r.px = (float)p[0];
  r.py = (float)p[1];
  r.pz = (float)p[2];
  r.dx = (float)d[0];
  r.dy = (float)d[1];
  r.dz = (float)d[2];
  r.lx = r.ly = r.lz = 0.f;
  unit_ff(r.dx, r.dy, r.dz, r.lx, r.ly, r.lz);
  r.wl = (float)reinterpret_cast<const double*>(s.wavelength)[i];
  r.inten = 1.f;
  r.att = 0.f;
  r.n = 1.f;
  r.ok = true;
  r.opl_hi = r.opl_lo = 0.f;
  for (int k = 0; k < sys.num_surfaces; ++k) propagate_surface<AnyKind, true>(sys, sys.surfaces[k], r);
  // system frame (the trace's output frame), then the last stop's frame
  float ox = r.px, oy = r.py, oz = r.pz;
  affine_point_folded(sys.final_to_output, ox, oy, oz);
  float ux = r.dx + r.lx, uy = r.dy + r.ly, uz = r.dz + r.lz;
  rotate(sys.final_to_output, ux, uy, uz);
  const double* T = s.to_last;  // 3 x 4 row-major
  const double v[3] = {s.target_direction ? (double)ux : (double)ox,
                       s.target_direction ? (double)uy : (double)oy,
                       s.target_direction ? (double)uz : (double)oz};
  const double w = s.target_direction ? 0.0 : 1.0;
  const double cx = fma(T[0], v[0], fma(T[1], v[1], fma(T[2], v[2], w * T[3])));
  const double cy = fma(T[4], v[0], fma(T[5], v[1], fma(T[6], v[2], w * T[7])));
  fx = cx - reinterpret_cast<const double*>(s.target_x)[i];
  fy = cy - reinterpret_cast<const double*>(s.target_y)[i];
}

__global__ void __launch_bounds__(128) k_stop_newton(const __grid_constant__ otx_system sys,
                                                     const __grid_constant__ StopArgs A) {
  const otx_stop_solve& s = A.s;
  const int64_t n = s.count;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  double* P = reinterpret_cast<double*>(s.position);
  double* D = reinterpret_cast<double*>(s.direction);
  int32_t* status = reinterpret_cast<int32_t*>(s.status);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    double* V = s.free_position ? P : D;
    double x = V[i], y = V[n + i];
    const double h = s.step;
    int polish = -1, done = -1;
    for (int it = 0; it < s.max_iterations; ++it) {
      double f0x, f0y;
      stop_residual(sys, A, i, x, y, f0x, f0y);
      const double err = fmax(fabs(f0x), fabs(f0y));
      if (polish < 0 && err < s.tolerance) polish = s.polish_steps;
      if (polish == 0) {
        done = it;
        break;
      }
      double f1x, f1y, f2x, f2y;
      stop_residual(sys, A, i, x + h, y, f1x, f1y);
      stop_residual(sys, A, i, x, y + h, f2x, f2y);
      const double j11 = (f1x - f0x) / h, j21 = (f1y - f0y) / h;
      const double j12 = (f2x - f0x) / h, j22 = (f2y - f0y) / h;
      const double det = j11 * j22 - j12 * j21;
      if (isfinite(det) && det != 0.0) {
        x -= (j22 * f0x - j12 * f0y) / det;
        y -= (-j21 * f0x + j11 * f0y) / det;
      }
      if (polish > 0) --polish;
    }
    // the solved free component, its z from the sag or the unit length
    V[i] = x;
    V[n + i] = y;
    if (s.free_position) {
      float gx, gy;
      V[2 * n + i] = (double)sag_eval(A.first.sag_type, A.first, (float)x, (float)y, gx, gy);
    } else {
      V[2 * n + i] = sqrt(1.0 - (x * x + y * y));
    }
    status[i] = done;
  }
}

}  // namespace otx

using namespace otx;

extern "C" otx_status otx_stop_newton(const otx_system* sub, const otx_system* first_sag,
                                      const otx_stop_solve* solve, void* stream) {
  if (!sub || !first_sag || !solve) return OTX_ERR_INVALID;
  if (const otx_status vs = validate_system(sub)) return vs;
  if (first_sag->num_surfaces < 1) return OTX_ERR_INVALID;
  const otx_stop_solve& s = *solve;
  if (s.count < 0 || s.max_iterations < 1 || s.polish_steps < 0 || !(s.step != 0.0) ||
      !(s.tolerance > 0.0))
    return OTX_ERR_INVALID;
  if (s.count == 0) return OTX_OK;
  if (!s.position || !s.direction || !s.wavelength || !s.target_x || !s.target_y || !s.status)
    return OTX_ERR_INVALID;
  StopArgs A;
  memset(&A, 0, sizeof(A));
  A.s = s;
  A.first = first_sag->surfaces[0];
  const int block = 128;
  const int64_t need = (s.count + block - 1) / block;
  const int grid = (int)(need < 4096 ? need : 4096);
  k_stop_newton<<<grid, block, 0, reinterpret_cast<cudaStream_t>(stream)>>>(*sub, A);
  return cudaGetLastError() == cudaSuccess ? OTX_OK : OTX_ERR_CUDA;
}
