// Building blocks of the tangent-linear and adjoint RK2 step: pointwise
// operators on groups of three spectral fields and on three real physical
// fields.  The step algebra itself is composed on the host (gt_tl_adj.cu).
//
// Inner products.  Spectral fields represent real fields; the adjoint is
// taken with respect to <x, y> = sum over stored modes of w_k Re(conj(x_k) y_k),
// w = 1 on the kx = 0 and kx = NX/2 planes and 2 elsewhere (the full-spectrum
// sum), and physical fields with sum_x f(x) g(x).  Under these, curl, k^2,
// invcurl, trunc and emk are self-adjoint, the Coriolis factor i omega kz has
// adjoint -i omega kz, fft_dir^T = fft_inv / (NX NY NZ) and
// fft_inv^T = (NX NY NZ) fft_dir.
#include "gt_fft.cuh"
#include "gt_internal.h"

namespace gt {

namespace {

struct P3 {
  void* p[3];
};

template <typename R>
__device__ __forceinline__ void kvec(const DevTables<R>& tb, int X, int y, int z, R& kx, R& ky, R& kz) {
  kx = tb.fkx[X];
  ky = tb.fky[y];
  kz = tb.fkz[z];
}

// out = op(a) (+ beta * b when accumulate), over all stored modes.
//  op 0: curl a = i k x a                   op 1: k^2 a
//  op 2: invcurl a (k = 0 left as is)       op 3: trunc (mask; k = 0 -> 0)
//  op 4: i*sgn*omega*kz a                   op 5: emk a
//  op 6: a (copy / axpy)                    op 7: 1{|k| >= kmin} a
//  op 8: a with the k = 0 mode set to 0
template <typename R>
__global__ void k_spec_op(P3 out, P3 a, P3 b, DevTables<R> tb, Geom g, int op, R sgn, R kmin2, R beta,
                          int accumulate) {
  using C = Cplx<R>;
  const size_t rows = (size_t)g.ny * g.nz;
  for (size_t row = blockIdx.y; row < rows; row += gridDim.y) {
    const int y = (int)(row % g.ny), z = (int)(row / g.ny);
    for (int X = blockIdx.x * blockDim.x + threadIdx.x; X < g.nh; X += gridDim.x * blockDim.x) {
      const size_t o = row * g.nhp + X;
      C v[3];
      for (int c = 0; c < 3; ++c) v[c] = reinterpret_cast<const C*>(a.p[c])[o];
      R kx, ky, kz;
      kvec(tb, X, y, z, kx, ky, kz);
      const R k2 = (tb.fkxs[X] + tb.fkys[y]) + tb.fkzs[z];
      const bool zero_mode = (X == 0) && (y == 0) && (z == 0);
      C r[3];
      switch (op) {
        case 0:
          r[0] = C{-ky * v[2].y + kz * v[1].y, ky * v[2].x - kz * v[1].x};
          r[1] = C{-kz * v[0].y + kx * v[2].y, kz * v[0].x - kx * v[2].x};
          r[2] = C{-kx * v[1].y + ky * v[0].y, kx * v[1].x - ky * v[0].x};
          break;
        case 1:
          for (int c = 0; c < 3; ++c) r[c] = C{k2 * v[c].x, k2 * v[c].y};
          break;
        case 2:
          if (zero_mode) {
            for (int c = 0; c < 3; ++c) r[c] = v[c];
          } else {
            const R qx = kx / k2, qy = ky / k2, qz = kz / k2;
            r[0] = C{-qy * v[2].y + qz * v[1].y, qy * v[2].x - qz * v[1].x};
            r[1] = C{-qz * v[0].y + qx * v[2].y, qz * v[0].x - qx * v[2].x};
            r[2] = C{-qx * v[1].y + qy * v[0].y, qx * v[1].x - qy * v[0].x};
          }
          break;
        case 3: {
          const bool kill = tb.truncate && (zero_mode || X >= tb.xcut[(size_t)z * g.ny + y]);
          for (int c = 0; c < 3; ++c) r[c] = kill ? C{0, 0} : v[c];
          break;
        }
        case 4: {
          const R f = sgn * tb.omega * kz;   // i f v = (-f v.y, f v.x)
          for (int c = 0; c < 3; ++c) r[c] = C{-f * v[c].y, f * v[c].x};
          break;
        }
        case 5: {
          const R e = tb.emk_by_k2 ? tb.emk[(int)k2] : tb.emk[((size_t)z * g.ny + y) * g.nh + X];
          for (int c = 0; c < 3; ++c) r[c] = C{e * v[c].x, e * v[c].y};
          break;
        }
        case 7: {
          const bool keep = k2 >= kmin2;
          for (int c = 0; c < 3; ++c) r[c] = keep ? v[c] : C{0, 0};
          break;
        }
        case 8:
          for (int c = 0; c < 3; ++c) r[c] = zero_mode ? C{0, 0} : v[c];
          break;
        default:
          for (int c = 0; c < 3; ++c) r[c] = v[c];
      }
      for (int c = 0; c < 3; ++c) {
        C* po = reinterpret_cast<C*>(out.p[c]);
        if (accumulate) {
          const C w = reinterpret_cast<const C*>(b.p[c])[o];
          po[o] = C{r[c].x + beta * w.x, r[c].y + beta * w.y};
        } else {
          po[o] = r[c];
        }
      }
    }
  }
}

// out = s1 * (a x b) + s2 * (c x d) on real fields (d, c may be null).
template <typename R>
__global__ void k_phys_cross(P3 out, P3 a, P3 b, P3 c, P3 d, R s1, R s2, int two, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const R a0 = reinterpret_cast<const R*>(a.p[0])[i], a1 = reinterpret_cast<const R*>(a.p[1])[i],
            a2 = reinterpret_cast<const R*>(a.p[2])[i];
    const R b0 = reinterpret_cast<const R*>(b.p[0])[i], b1 = reinterpret_cast<const R*>(b.p[1])[i],
            b2 = reinterpret_cast<const R*>(b.p[2])[i];
    R r0 = s1 * (a1 * b2 - a2 * b1), r1 = s1 * (a2 * b0 - a0 * b2), r2 = s1 * (a0 * b1 - a1 * b0);
    if (two) {
      const R c0 = reinterpret_cast<const R*>(c.p[0])[i], c1 = reinterpret_cast<const R*>(c.p[1])[i],
              c2 = reinterpret_cast<const R*>(c.p[2])[i];
      const R d0 = reinterpret_cast<const R*>(d.p[0])[i], d1 = reinterpret_cast<const R*>(d.p[1])[i],
              d2 = reinterpret_cast<const R*>(d.p[2])[i];
      r0 += s2 * (c1 * d2 - c2 * d1);
      r1 += s2 * (c2 * d0 - c0 * d2);
      r2 += s2 * (c0 * d1 - c1 * d0);
    }
    reinterpret_cast<R*>(out.p[0])[i] = r0;
    reinterpret_cast<R*>(out.p[1])[i] = r1;
    reinterpret_cast<R*>(out.p[2])[i] = r2;
  }
}

}  // namespace

template <typename R>
int launch_spec_op(const Geom& g, const DevTables<R>& tb, void* const out[3], void* const a[3],
                   void* const b[3], int op, double sgn, double kmin2, double beta, void* stream) {
  P3 po{}, pa{}, pb{};
  for (int c = 0; c < 3; ++c) {
    po.p[c] = out[c];
    pa.p[c] = a[c];
    pb.p[c] = b ? b[c] : a[c];
  }
  const int threads = 128;
  const int bx = (g.nh + threads - 1) / threads;
  const int by = (int)std::min<long long>((long long)g.ny * g.nz, 65535);
  k_spec_op<R><<<dim3(bx, by), threads, 0, (cudaStream_t)stream>>>(po, pa, pb, tb, g, op, (R)sgn, (R)kmin2,
                                                                    (R)beta, b ? 1 : 0);
  return (int)cudaGetLastError();
}

template <typename R>
int launch_phys_cross(const Geom& g, void* const out[3], void* const a[3], void* const b[3],
                      void* const c[3], void* const d[3], double s1, double s2, void* stream) {
  P3 po{}, pa{}, pb{}, pc{}, pd{};
  for (int i = 0; i < 3; ++i) {
    po.p[i] = out[i];
    pa.p[i] = a[i];
    pb.p[i] = b[i];
    pc.p[i] = c ? c[i] : a[i];
    pd.p[i] = d ? d[i] : b[i];
  }
  const size_t n = (size_t)g.nx * g.ny * g.nz;
  const int threads = 256;
  const int blocks = (int)std::min<size_t>((n + threads - 1) / threads, 152 * 16);
  k_phys_cross<R><<<blocks, threads, 0, (cudaStream_t)stream>>>(po, pa, pb, pc, pd, (R)s1, (R)s2,
                                                                 c != nullptr, n);
  return (int)cudaGetLastError();
}

template int launch_spec_op<float>(const Geom&, const DevTables<float>&, void* const*, void* const*,
                                   void* const*, int, double, double, double, void*);
template int launch_spec_op<double>(const Geom&, const DevTables<double>&, void* const*, void* const*,
                                    void* const*, int, double, double, double, void*);
template int launch_phys_cross<float>(const Geom&, void* const*, void* const*, void* const*, void* const*,
                                      void* const*, double, double, void*);
template int launch_phys_cross<double>(const Geom&, void* const*, void* const*, void* const*, void* const*,
                                       void* const*, double, double, void*);

}  // namespace gt
