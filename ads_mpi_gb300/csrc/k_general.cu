// k_general.cu — FP64 kernels for a general geometry: a separate degree per
// axis, as initialize(n(3), p(3), ...) allows (src/ADS.F90:11, the per-axis
// p of ADS_setup in src/Setup.F90:29-140).
//
// The tuned kernels (k_assemble*, k_residual, k_sweep, k_csweep) take one
// degree as a template parameter and size their tiles by it.  These kernels
// take the three degrees at run time instead, with the element's coefficient
// block and its local right-hand side in per-thread arrays of at most 5^3
// entries, and favour simplicity over speed:
//   k_assemble_gen   FormUn + Form3DRHS (src/projection_engine.F90:154-441)
//                    with the projection and heat integrands; one thread per
//                    element of one colour class (element e has colour
//                    e mod (p+1) per axis, so elements of a class share no
//                    DOF: the scatter needs no atomics and the order in which
//                    each DOF receives its element parts is fixed)
//   k_residual_gen   r = F - (Mx (x) My (x) Mz) u, one thread per DOF
//   k_kappa_grad_gen dL/dkappa at the quadrature points (the adjoint)
//   k_permute        ReorderRHSForY/Z/X (src/reorderRHS.F90:7-93)
#include "ads_internal.cuh"

namespace ads {

constexpr int GEN_THREADS = 128;
constexpr int GEN_MAXB = 125;  // (p+1)^3 entries of an element block, p <= 4

static long long gen_colour_elems(const Geometry& g) {
  long long n = 1;
  for (int d = 0; d < 3; ++d) n *= (g.E[d] + g.p[d]) / (g.p[d] + 1);  // ceil(E / (p+1))
  return n;
}

static int gen_colour_blocks(const Geometry& g) {
  return (int)((gen_colour_elems(g) + GEN_THREADS - 1) / GEN_THREADS);
}

long long assemble_gen_parts(const Geometry& g) {
  return (long long)(g.p[0] + 1) * (g.p[1] + 1) * (g.p[2] + 1) * gen_colour_blocks(g);
}

__global__ void __launch_bounds__(GEN_THREADS) k_assemble_gen(const GenAssembleArgs a, int cx, int cy, int cz,
                                                               int colour) {
  const Geometry& g = a.g;
  const int px = g.p[0], py = g.p[1], pz = g.p[2];
  const int qx = g.q[0], qy = g.q[1], qz = g.q[2];
  const int sx = px + 1, sy = py + 1, sz = pz + 1;
  const int nx = (g.E[0] - cx + sx - 1) / sx, ny = (g.E[1] - cy + sy - 1) / sy, nz = (g.E[2] - cz + sz - 1) / sz;
  const long long nel = (long long)nx * ny * nz;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool heat = a.form == ADS_FORM_HEAT;
  double l2 = 0.0;
  if (t < nel) {
    const int ex = cx + sx * (int)(t % nx);
    const int ey = cy + sy * (int)((t / nx) % ny);
    const int ez = cz + sz * (int)(t / ((long long)nx * ny));
    const int Ny = g.N[1];
    double c[GEN_MAXB], fl[GEN_MAXB];
    for (int bz = 0; bz < sz; ++bz)
      for (int by = 0; by < sy; ++by)
        for (int bx = 0; bx < sx; ++bx) {
          const int i = (bz * sy + by) * sx + bx;
          c[i] = heat ? a.u[(size_t)(ex + bx) + (size_t)g.PX * ((size_t)(ey + by) + (size_t)Ny * (ez + bz))] : 0.0;
          fl[i] = 0.0;
        }
    const double* NX = a.nn[0] + (size_t)ex * qx * sx * 2;
    const double* NY = a.nn[1] + (size_t)ey * qy * sy * 2;
    const double* NZ = a.nn[2] + (size_t)ez * qz * sz * 2;
    const double* JX = a.jw[0] + (size_t)ex * qx;
    const double* JY = a.jw[1] + (size_t)ey * qy;
    const double* JZ = a.jw[2] + (size_t)ez * qz;
    const long long QX = (long long)g.E[0] * qx, QY = (long long)g.E[1] * qy;
    for (int kz = 0; kz < qz; ++kz)
      for (int ky = 0; ky < qy; ++ky)
        for (int kx = 0; kx < qx; ++kx) {
          const double w = JX[kx] * JY[ky] * JZ[kz];
          const long long gi = ((long long)ex * qx + kx) + QX * (((long long)ey * qy + ky) + QY * ((long long)ez * qz + kz));
          const double f = a.fqp ? a.fqp[gi] : (heat ? 0.0 : 1.0);
          double g0, g1 = 0.0, g2 = 0.0, g3 = 0.0;
          if (heat) {
            // u and grad u at the point, summed over x first, then y, then z
            double uu = 0.0, dx = 0.0, dy = 0.0, dz = 0.0;
            for (int bz = 0; bz < sz; ++bz) {
              double a0 = 0.0, a1 = 0.0, a2 = 0.0;
              for (int by = 0; by < sy; ++by) {
                double s0 = 0.0, s1 = 0.0;
                for (int bx = 0; bx < sx; ++bx) {
                  const double cv = c[(bz * sy + by) * sx + bx];
                  s0 += NX[(kx * sx + bx) * 2 + 0] * cv;
                  s1 += NX[(kx * sx + bx) * 2 + 1] * cv;
                }
                const double nyv = NY[(ky * sy + by) * 2 + 0], nyd = NY[(ky * sy + by) * 2 + 1];
                a0 += nyv * s0;
                a1 += nyv * s1;
                a2 += nyd * s0;
              }
              const double nzv = NZ[(kz * sz + bz) * 2 + 0], nzd = NZ[(kz * sz + bz) * 2 + 1];
              uu += nzv * a0;
              dx += nzv * a1;
              dy += nzv * a2;
              dz += nzd * a0;
            }
            const double kq = a.kqp ? a.kqp[gi] : a.kappa;
            const double ck = -a.dt * kq * w;
            g0 = a.incr ? w * a.dt * f : w * (uu + a.dt * f);
            g1 = ck * dx;
            g2 = ck * dy;
            g3 = ck * dz;
            l2 += w * uu * uu;
          } else {
            g0 = w * f;
            l2 += w * f * f;
          }
          // test functions: F_a += g0 v_a + g1 dv_a/dx + g2 dv_a/dy + g3 dv_a/dz
          for (int az = 0; az < sz; ++az) {
            const double nzv = NZ[(kz * sz + az) * 2 + 0], nzd = NZ[(kz * sz + az) * 2 + 1];
            for (int ay = 0; ay < sy; ++ay) {
              const double nyv = NY[(ky * sy + ay) * 2 + 0], nyd = NY[(ky * sy + ay) * 2 + 1];
              const double t0 = g0 * nyv * nzv + g2 * nyd * nzv + g3 * nyv * nzd;
              const double t1 = g1 * nyv * nzv;
              for (int ax = 0; ax < sx; ++ax)
                fl[(az * sy + ay) * sx + ax] += NX[(kx * sx + ax) * 2 + 0] * t0 + NX[(kx * sx + ax) * 2 + 1] * t1;
            }
          }
        }
    for (int bz = 0; bz < sz; ++bz)
      for (int by = 0; by < sy; ++by)
        for (int bx = 0; bx < sx; ++bx)
          a.F[(size_t)(ex + bx) + (size_t)g.PX * ((size_t)(ey + by) + (size_t)Ny * (ez + bz))] +=
              fl[(bz * sy + by) * sx + bx];
  }
  // fixed-order block sum of the l2 partials
  __shared__ double red[GEN_THREADS];
  red[threadIdx.x] = l2;
  __syncthreads();
  for (int w = GEN_THREADS / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.part[(size_t)colour * gridDim.x + blockIdx.x] = red[0];
}

__global__ void k_gen_l2_final(const double* part, long long n, double* scal) {
  double t = 0.0;
  for (long long i = threadIdx.x; i < n; i += 32) t += part[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  if (threadIdx.x == 0) scal[SC_L2] = t;
}

cudaError_t launch_assemble_gen(const GenAssembleArgs& a, double* scal, cudaStream_t s) {
  const Geometry& g = a.g;
  for (int d = 0; d < 3; ++d)
    if (g.p[d] < 1 || g.p[d] > 4) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(a.F, 0, sizeof(double) * (size_t)g.PX * g.N[1] * g.N[2], s);
  if (e != cudaSuccess) return e;
  const int blocks = gen_colour_blocks(g);
  int colour = 0;
  for (int cz = 0; cz <= g.p[2]; ++cz)
    for (int cy = 0; cy <= g.p[1]; ++cy)
      for (int cx = 0; cx <= g.p[0]; ++cx, ++colour) {
        k_assemble_gen<<<blocks, GEN_THREADS, 0, s>>>(a, cx, cy, cz, colour);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
      }
  k_gen_l2_final<<<1, 32, 0, s>>>(a.part, assemble_gen_parts(g), scal);
  return cudaGetLastError();
}

__global__ void k_residual_gen(const Geometry g, const double* __restrict__ u, const double* __restrict__ F,
                               double* __restrict__ r, const double* __restrict__ bx, const double* __restrict__ by,
                               const double* __restrict__ bz) {
  const int Nx = g.N[0], Ny = g.N[1], Nz = g.N[2];
  const int px = g.p[0], py = g.p[1], pz = g.p[2];
  const long long n = (long long)Nx * Ny * Nz;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i % Nx), y = (int)((i / Nx) % Ny), z = (int)(i / ((long long)Nx * Ny));
    double sum = 0.0;
    for (int mz = -pz; mz <= pz; ++mz) {
      if (z + mz < 0 || z + mz >= Nz) continue;
      double sy = 0.0;
      for (int my = -py; my <= py; ++my) {
        if (y + my < 0 || y + my >= Ny) continue;
        const double* row = u + (size_t)g.PX * ((size_t)(y + my) + (size_t)Ny * (z + mz));
        double sx = 0.0;
        for (int mx = -px; mx <= px; ++mx) {
          if (x + mx < 0 || x + mx >= Nx) continue;
          sx += bx[(size_t)(mx + px) * Nx + x] * row[x + mx];
        }
        sy += by[(size_t)(my + py) * Ny + y] * sx;
      }
      sum += bz[(size_t)(mz + pz) * Nz + z] * sy;
    }
    const size_t o = (size_t)x + (size_t)g.PX * ((size_t)y + (size_t)Ny * z);
    r[o] = F ? F[o] - sum : sum;
  }
}

cudaError_t launch_residual_gen(const Geometry& g, const double* u, const double* F, double* r,
                                const double* const band[3], cudaStream_t s) {
  const long long n = (long long)g.N[0] * g.N[1] * g.N[2];
  long long b = (n + 255) / 256;
  if (b > 152 * 64) b = 152 * 64;
  k_residual_gen<<<(int)b, 256, 0, s>>>(g, u, F, r, band[0], band[1], band[2]);
  return cudaGetLastError();
}

// -dt J W grad u(q) . grad mu(q), accumulated at every quadrature point; one
// thread per element (elements own their points, so no two threads share one)
__global__ void k_kappa_grad_gen(const Geometry g, const double* __restrict__ u, const double* __restrict__ mu,
                                 double dt, double* gk, AxisTab<double> tx, AxisTab<double> ty, AxisTab<double> tz) {
  const int px = g.p[0], py = g.p[1], pz = g.p[2];
  const int qx = g.q[0], qy = g.q[1], qz = g.q[2];
  const int sx = px + 1, sy = py + 1, sz = pz + 1;
  const long long Ex = g.E[0], Ey = g.E[1], Ez = g.E[2];
  const long long QX = Ex * qx, QY = Ey * qy;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < Ex * Ey * Ez;
       e += (long long)gridDim.x * blockDim.x) {
    const long long ex = e % Ex, ey = (e / Ex) % Ey, ez = e / (Ex * Ey);
    double cu[GEN_MAXB], cm[GEN_MAXB];
    for (int c = 0; c < sz; ++c)
      for (int b = 0; b < sy; ++b)
        for (int a = 0; a < sx; ++a) {
          const size_t o = (size_t)(ex + a) + (size_t)g.PX * ((size_t)(ey + b) + (size_t)g.N[1] * (size_t)(ez + c));
          cu[(c * sy + b) * sx + a] = u[o];
          cm[(c * sy + b) * sx + a] = mu[o];
        }
    for (int kz = 0; kz < qz; ++kz)
      for (int ky = 0; ky < qy; ++ky)
        for (int kx = 0; kx < qx; ++kx) {
          double gu[3] = {0.0, 0.0, 0.0}, gm[3] = {0.0, 0.0, 0.0};
          for (int c = 0; c < sz; ++c) {
            const double nz0 = tz.nn[((ez * qz + kz) * sz + c) * 2 + 0];
            const double nz1 = tz.nn[((ez * qz + kz) * sz + c) * 2 + 1];
            for (int b = 0; b < sy; ++b) {
              const double ny0 = ty.nn[((ey * qy + ky) * sy + b) * 2 + 0];
              const double ny1 = ty.nn[((ey * qy + ky) * sy + b) * 2 + 1];
              for (int a = 0; a < sx; ++a) {
                const double nx0 = tx.nn[((ex * qx + kx) * sx + a) * 2 + 0];
                const double nx1 = tx.nn[((ex * qx + kx) * sx + a) * 2 + 1];
                const double wx = nx1 * ny0 * nz0, wy = nx0 * ny1 * nz0, wz = nx0 * ny0 * nz1;
                const double vu = cu[(c * sy + b) * sx + a], vm = cm[(c * sy + b) * sx + a];
                gu[0] += wx * vu; gu[1] += wy * vu; gu[2] += wz * vu;
                gm[0] += wx * vm; gm[1] += wy * vm; gm[2] += wz * vm;
              }
            }
          }
          const double jw = tx.jw[ex * qx + kx] * ty.jw[ey * qy + ky] * tz.jw[ez * qz + kz];
          const long long gi = (ex * qx + kx) + QX * ((ey * qy + ky) + QY * (ez * qz + kz));
          gk[gi] += -dt * jw * (gu[0] * gm[0] + gu[1] * gm[1] + gu[2] * gm[2]);
        }
  }
}

cudaError_t launch_kappa_grad_gen(const Geometry& g, const double* u, const double* mu, double dt, double* gk,
                                  const AxisTab<double>& tx, const AxisTab<double>& ty, const AxisTab<double>& tz,
                                  cudaStream_t s) {
  const long long ne = (long long)g.E[0] * g.E[1] * g.E[2];
  long long b = (ne + 127) / 128;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  k_kappa_grad_gen<<<(int)b, 128, 0, s>>>(g, u, mu, dt, gk, tx, ty, tz);
  return cudaGetLastError();
}

// dense in -> dense out: FOR_Y  F(x, y+z*Ny)   -> F2(y, x+z*Nx)
//                         FOR_Z  F2(y, x+z*Nx) -> F3(z, x+y*Nx)
//                         FOR_X  F3(z, x+y*Nx) -> F(x, y+z*Ny)
__global__ void k_permute(const double* __restrict__ in, double* __restrict__ out, int Nx, int Ny, int Nz, int kind) {
  const long long n = (long long)Nx * Ny * Nz;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    long long j;
    if (kind == ADS_REORDER_FOR_Y) {  // i = x + Nx (y + Ny z)
      const long long x = i % Nx, y = (i / Nx) % Ny, z = i / ((long long)Nx * Ny);
      j = y + (long long)Ny * (x + (long long)Nx * z);
    } else if (kind == ADS_REORDER_FOR_Z) {  // i = y + Ny (x + Nx z)
      const long long y = i % Ny, x = (i / Ny) % Nx, z = i / ((long long)Ny * Nx);
      j = z + (long long)Nz * (x + (long long)Nx * y);
    } else {  // i = z + Nz (x + Nx y)
      const long long z = i % Nz, x = (i / Nz) % Nx, y = i / ((long long)Nz * Nx);
      j = x + (long long)Nx * (y + (long long)Ny * z);
    }
    out[j] = in[i];
  }
}

cudaError_t launch_permute(const double* in, double* out, const Geometry& g, int kind, cudaStream_t s) {
  const long long n = (long long)g.N[0] * g.N[1] * g.N[2];
  long long b = (n + 255) / 256;
  if (b > 152 * 64) b = 152 * 64;
  k_permute<<<(int)b, 256, 0, s>>>(in, out, g.N[0], g.N[1], g.N[2], kind);
  return cudaGetLastError();
}

}  // namespace ads
