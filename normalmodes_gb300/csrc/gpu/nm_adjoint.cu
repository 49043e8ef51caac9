// nm_adjoint: eigenvalue sensitivities to the per-element material,
//   dlam/dm_e = z^T (dK/dm_e - lam dM/dm_e) z,   z = [x; p],
// for m = density, bulk modulus, shear modulus (the other two fixed), where
// dm_e shifts every nodal value of m in element e by the same amount.
//
// The element matrices of the reference's CG mixed FEM (CGE3D_ISO /
// CGFSE3D_ISO, src/mod_cg_create_matrix.f90:103-1266, JOB = 1) are linear
// in the nodal Lame lambda, mu and density, so for a uniform shift the
// derivative matrices are the element matrices with unit coefficients:
//   solid stiffness, lambda = 1:   sum_ij (D_i u_i)^T M (D_j u_j) detJ
//                    = div^T M div detJ
//   solid stiffness, mu = 1:        2 sum_ik eps_ik^T M eps_ik detJ,
//                    eps_ik = (D_k u_i + D_i u_k) / 2
//   mass, rho = 1:                  sum_i u_i^T M u_i detJ
// (D_k = sum_j invJ[k][j] Dr_j the nodal derivative matrices, M the
// reference mass), and bulk / shear at fixed other parameter follow from
// lambda = kappa - 2 mu / 3.  In a fluid element the material enters only
// the pressure block -detJ diag(lambda^-1/2) M diag(lambda^-1/2) (:453-640),
// whose derivative for a uniform shift of lambda = kappa gives
//   dlam/dkappa_e = detJ (p .* lambda^-3/2)^T M (p .* lambda^-1/2).
// Each thread recomputes its element's geometry and nodal fields for one
// eigenvector; nothing per element is stored.  With the reference gravity
// (JOB = 2) the host adds the gravity terms (nm_adjoint_gravity).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "nm_internal.h"

namespace nmg {
namespace {

constexpr int kTA = 128;

template <int P>
__device__ __forceinline__ double qform(const double* sM, const double* x, const double* y) {
  double s = 0.0;
#pragma unroll
  for (int a = 0; a < P; ++a) {
    double t = 0.0;
#pragma unroll
    for (int b = 0; b < P; ++b) t = fma(sM[a * P + b], y[b], t);
    s = fma(x[a], t, s);
  }
  return s;
}

template <int P>
__global__ void __launch_bounds__(kTA)
    k_adjoint(int ntet, int kc, int n, int np, const int* __restrict__ tets, const double* __restrict__ xyz,
              const unsigned char* __restrict__ fluid, const int* __restrict__ vstt, const int* __restrict__ rnum,
              const int* __restrict__ pstt, const double* __restrict__ lamf, const double* __restrict__ refM,
              const double* __restrict__ refD, int4 vord, const double* __restrict__ X,
              const double* __restrict__ Pp, const double* __restrict__ lam, double* __restrict__ grad) {
  __shared__ double sM[P * P], sD[3 * P * P];
  for (int i = threadIdx.x; i < P * P; i += blockDim.x) sM[i] = refM[i];
  for (int i = threadIdx.x; i < 3 * P * P; i += blockDim.x) sD[i] = refD[i];
  __syncthreads();
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (long long)ntet * kc) return;
  const int j = (int)(tid / ntet), e = (int)(tid % ntet);
  const int* nodes = tets + (size_t)e * P;
  // geometry: rows of Bm are x_v - x_0; invJ = 2 Bm^-1, detJ = det(Bm) / 8
  double x0[3], Bm[3][3];
  {
    const int v[4] = {vord.x, vord.y, vord.z, vord.w};
    for (int c = 0; c < 3; ++c) x0[c] = xyz[3 * (size_t)nodes[v[0]] + c];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) Bm[r][c] = xyz[3 * (size_t)nodes[v[r + 1]] + c] - x0[c];
  }
  const double det = Bm[0][0] * (Bm[1][1] * Bm[2][2] - Bm[1][2] * Bm[2][1]) -
                     Bm[0][1] * (Bm[1][0] * Bm[2][2] - Bm[1][2] * Bm[2][0]) +
                     Bm[0][2] * (Bm[1][0] * Bm[2][1] - Bm[1][1] * Bm[2][0]);
  const double detJ = det / 8.0;
  double invJ[3][3];
  {
    const double s = 2.0 / det;
    invJ[0][0] = s * (Bm[1][1] * Bm[2][2] - Bm[1][2] * Bm[2][1]);
    invJ[0][1] = s * (Bm[0][2] * Bm[2][1] - Bm[0][1] * Bm[2][2]);
    invJ[0][2] = s * (Bm[0][1] * Bm[1][2] - Bm[0][2] * Bm[1][1]);
    invJ[1][0] = s * (Bm[1][2] * Bm[2][0] - Bm[1][0] * Bm[2][2]);
    invJ[1][1] = s * (Bm[0][0] * Bm[2][2] - Bm[0][2] * Bm[2][0]);
    invJ[1][2] = s * (Bm[0][2] * Bm[1][0] - Bm[0][0] * Bm[1][2]);
    invJ[2][0] = s * (Bm[1][0] * Bm[2][1] - Bm[1][1] * Bm[2][0]);
    invJ[2][1] = s * (Bm[0][1] * Bm[2][0] - Bm[0][0] * Bm[2][1]);
    invJ[2][2] = s * (Bm[0][0] * Bm[1][1] - Bm[0][1] * Bm[1][0]);
  }
  const bool fl = fluid[e] != 0;
  const double* x = X + (size_t)j * n;
  double u[3][P];
#pragma unroll
  for (int a = 0; a < P; ++a) {
    const int nd = nodes[a];
    const int base = vstt[nd] + (fl ? rnum[nd] - 3 : 0);
#pragma unroll
    for (int i = 0; i < 3; ++i) u[i][a] = x[base + i];
  }
  double qm = 0.0;
#pragma unroll
  for (int i = 0; i < 3; ++i) qm += qform<P>(sM, u[i], u[i]);
  double g_rho = -lam[j] * detJ * qm, g_kappa = 0.0, g_mu = 0.0;
  if (!fl) {
    // G[k][i][a] = (D_k u_i)[a]
    double G[3][3][P];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int a = 0; a < P; ++a) {
        double w[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int b = 0; b < P; ++b) w[d] = fma(sD[(d * P + a) * P + b], u[i][b], w[d]);
#pragma unroll
        for (int k = 0; k < 3; ++k) G[k][i][a] = invJ[k][0] * w[0] + invJ[k][1] * w[1] + invJ[k][2] * w[2];
      }
    double div[P];
#pragma unroll
    for (int a = 0; a < P; ++a) div[a] = G[0][0][a] + G[1][1][a] + G[2][2][a];
    const double qdiv = qform<P>(sM, div, div);
    double qeps = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        double ek[P];
#pragma unroll
        for (int a = 0; a < P; ++a) ek[a] = 0.5 * (G[k][i][a] + G[i][k][a]);
        qeps += qform<P>(sM, ek, ek);
      }
    g_kappa = detJ * qdiv;
    g_mu = detJ * (2.0 * qeps - (2.0 / 3.0) * qdiv);
  } else if (Pp) {
    const double* pj = Pp + (size_t)j * np;
    double pa[P], pb[P];
#pragma unroll
    for (int a = 0; a < P; ++a) {
      const double l = lamf[(size_t)e * P + a];
      const double pv = pj[pstt[nodes[a]]];
      const double ri = rsqrt(l);
      pb[a] = pv * ri;
      pa[a] = pv * ri / l;
    }
    g_kappa = detJ * qform<P>(sM, pa, pb);
  }
  double* o = grad + ((size_t)j * ntet + e) * 3;
  o[0] = g_rho;
  o[1] = g_kappa;
  o[2] = g_mu;
}

__global__ void k_div(const double* __restrict__ x, const double* __restrict__ d, double* __restrict__ y, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] / d[i];
}
__global__ void k_mul(const double* __restrict__ x, const double* __restrict__ d, double* __restrict__ y, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] * d[i];
}

template <typename T>
int dev_copy(nm_ctx* c, T** d, const T* h, size_t cnt, std::vector<void*>& owned) {
  NM_CUDA(c, cudaMalloc((void**)d, sizeof(T) * std::max<size_t>(cnt, 1)));
  owned.push_back(*d);
  if (cnt) NM_CUDA(c, cudaMemcpyAsync(*d, h, sizeof(T) * cnt, cudaMemcpyHostToDevice, c->stream));
  return NM_OK;
}

}  // namespace
}  // namespace nmg

using namespace nmg;

int nm_adjoint(nm_ctx* c, const nm_elem_model* em, int k, const double* lam, const double* X, int ldx, int mode,
               double tol, double* grad, int* group, int* ngroups) {
  if (!c) return NM_ERR_ARG;
  if (!em || !lam || !X || !grad || k < 0 || ldx < c->n)
    return set_err(c, NM_ERR_ARG, "nm_adjoint: bad arguments");
  if (mode != NM_ADJ_PAIR && mode != NM_ADJ_MULTIPLET) return set_err(c, NM_ERR_ARG, "nm_adjoint: bad mode");
  const int P = em->pnp, ntet = em->ntet, n = c->n, np = c->np;
  if (P != 4 && P != 10) return set_err(c, NM_ERR_ARG, "nm_adjoint: pnp must be 4 (P1) or 10 (P2)");
  if ((em->fluid_solid != 0) != (c->fs != 0))
    return set_err(c, NM_ERR_ARG, "nm_adjoint: element model and operators disagree on the fluid-solid split");
  if (!em->tets || !em->xyz || !em->fluid || !em->vstt || !em->rnum || !em->vp || !em->vs || !em->rho ||
      !em->ref_mass || !em->ref_drst || (c->fs && !em->pstt))
    return set_err(c, NM_ERR_ARG, "nm_adjoint: missing element-model array");
  if (em->g0 && (!em->ref_massf || !em->ref_fmask))
    return set_err(c, NM_ERR_ARG, "nm_adjoint: gravity terms need the reference face masses and face lists");
  // every DOF the elements address must exist
  for (int e = 0; e < ntet; ++e)
    for (int a = 0; a < P; ++a) {
      const int nd = em->tets[(size_t)e * P + a];
      if (nd < 0 || nd >= em->nnode) return set_err(c, NM_ERR_ARG, "nm_adjoint: node index out of range");
      const int rn = em->rnum[nd];
      if ((rn != 3 && rn != 6) || em->vstt[nd] < 0 || em->vstt[nd] + rn > n)
        return set_err(c, NM_ERR_ARG, "nm_adjoint: displacement DOF out of range");
      if (em->fluid[e] && c->fs && (em->pstt[nd] < 0 || em->pstt[nd] >= np))
        return set_err(c, NM_ERR_ARG, "nm_adjoint: pressure DOF out of range");
    }
  if (ngroups) *ngroups = 0;
  if (k == 0 || ntet == 0) return NM_OK;
  if (cudaSetDevice(c->device) != cudaSuccess) return set_err(c, NM_ERR_CUDA, "cudaSetDevice failed");
  cudaStream_t s = c->stream;
  // nodal Lame lambda (the fluid bulk modulus) of every element node
  std::vector<double> lamf((size_t)P * ntet);
  for (size_t q = 0; q < lamf.size(); ++q) {
    const double mu = em->rho[q] * em->vs[q] * em->vs[q];
    lamf[q] = em->rho[q] * em->vp[q] * em->vp[q] - 2.0 * mu;
  }
  const int4 vord = P == 4 ? make_int4(0, 1, 2, 3) : make_int4(0, 2, 5, 9);
  const int kc = std::min(k, 16);
  std::vector<void*> owned;
  auto release = [&]() {
    cudaStreamSynchronize(s);
    for (void* p : owned) cudaFree(p);
    owned.clear();
  };
  auto guard = on_exit(release);
  int *d_tets, *d_vstt, *d_rnum, *d_pstt = nullptr;
  double *d_xyz, *d_lamf, *d_M, *d_D;
  unsigned char* d_fluid;
  int rc;
  std::vector<int> pst(em->pstt ? em->pstt : em->vstt, (em->pstt ? em->pstt : em->vstt) + em->nnode);
  if ((rc = dev_copy(c, &d_tets, em->tets, (size_t)P * ntet, owned)) ||
      (rc = dev_copy(c, &d_xyz, em->xyz, (size_t)3 * em->nnode, owned)) ||
      (rc = dev_copy(c, &d_fluid, em->fluid, (size_t)ntet, owned)) ||
      (rc = dev_copy(c, &d_vstt, em->vstt, (size_t)em->nnode, owned)) ||
      (rc = dev_copy(c, &d_rnum, em->rnum, (size_t)em->nnode, owned)) ||
      (rc = dev_copy(c, &d_pstt, pst.data(), pst.size(), owned)) ||
      (rc = dev_copy(c, &d_lamf, lamf.data(), lamf.size(), owned)) ||
      (rc = dev_copy(c, &d_M, em->ref_mass, (size_t)P * P, owned)) ||
      (rc = dev_copy(c, &d_D, em->ref_drst, (size_t)3 * P * P, owned))) {
    release();
    return rc;
  }
  double *dX = nullptr, *dP = nullptr, *dy = nullptr, *dt = nullptr, *dz = nullptr, *dwork = nullptr, *dlam = nullptr,
         *dg = nullptr;
  auto alloc = [&](double** p, size_t cnt) -> int {
    NM_CUDA(c, cudaMalloc((void**)p, sizeof(double) * std::max<size_t>(cnt, 1)));
    owned.push_back(*p);
    return NM_OK;
  };
  if ((rc = alloc(&dX, (size_t)n * kc)) || (rc = alloc(&dlam, kc)) || (rc = alloc(&dg, (size_t)kc * ntet * 3)) ||
      (c->fs && ((rc = alloc(&dP, (size_t)np * kc)) || (rc = alloc(&dy, n)) || (rc = alloc(&dt, np)) ||
                 (rc = alloc(&dz, np)) || (rc = alloc(&dwork, (size_t)4 * np))))) {
    release();
    return rc;
  }
  // per-pair gradients (host)
  std::vector<double> pair, hP;
  double* out_pairs = grad;
  if (mode == NM_ADJ_MULTIPLET) {
    pair.resize((size_t)k * ntet * 3);
    out_pairs = pair.data();
  }
  for (int j0 = 0; j0 < k; j0 += kc) {
    const int m = std::min(kc, k - j0);
    NM_CUDA(c, cudaMemcpy2DAsync(dX, sizeof(double) * n, X + (size_t)j0 * ldx, sizeof(double) * ldx,
                                 sizeof(double) * n, m, cudaMemcpyHostToDevice, s));
    NM_CUDA(c, cudaMemcpyAsync(dlam, lam + j0, sizeof(double) * m, cudaMemcpyHostToDevice, s));
    if (c->fs) {
      // p = (-Ap)^-1 ET x = D_p Cheb(Ap_s) ET_s (x ./ D)
      for (int jj = 0; jj < m; ++jj) {
        k_div<<<(n + 255) / 256, 256, 0, s>>>(dX + (size_t)jj * n, c->D, dy, n);
        spmv<double, double>(c->ET, dy, dt, s);
        cheb_solve<double, double>(c->Ap, c->chebAp, dt, dz, dwork, s);
        k_mul<<<(np + 255) / 256, 256, 0, s>>>(dz, c->Dp, dP + (size_t)jj * np, np);
        add_launches(4 + c->chebAp.deg);
      }
    }
    const long long threads = (long long)ntet * m;
    const int blocks = (int)((threads + kTA - 1) / kTA);
    if (P == 4)
      k_adjoint<4><<<blocks, kTA, 0, s>>>(ntet, m, n, np, d_tets, d_xyz, d_fluid, d_vstt, d_rnum, d_pstt, d_lamf, d_M,
                                          d_D, vord, dX, c->fs ? dP : nullptr, dlam, dg);
    else
      k_adjoint<10><<<blocks, kTA, 0, s>>>(ntet, m, n, np, d_tets, d_xyz, d_fluid, d_vstt, d_rnum, d_pstt, d_lamf,
                                           d_M, d_D, vord, dX, c->fs ? dP : nullptr, dlam, dg);
    add_launches(1);
    NM_CUDA(c, cudaGetLastError());
    NM_CUDA(c, cudaMemcpyAsync(out_pairs + (size_t)j0 * ntet * 3, dg, sizeof(double) * (size_t)m * ntet * 3,
                               cudaMemcpyDeviceToHost, s));
    if (em->g0 && c->fs) {
      hP.resize((size_t)np * m);
      NM_CUDA(c, cudaMemcpyAsync(hP.data(), dP, sizeof(double) * (size_t)np * m, cudaMemcpyDeviceToHost, s));
    }
    NM_CUDA(c, cudaStreamSynchronize(s));
    if (em->g0 && (rc = nm_adjoint_gravity(em, m, X + (size_t)j0 * ldx, ldx, c->fs ? hP.data() : nullptr, np,
                                           out_pairs + (size_t)j0 * ntet * 3))) {
      release();
      return set_err(c, rc, "nm_adjoint: gravity terms failed (degenerate element)");
    }
  }
  release();
  if ((rc = check_status(c))) return rc;
  // groups: runs of consecutive eigenvalues closer than tol (relative)
  std::vector<int> grp(k);
  int ng = 0;
  for (int i = 0; i < k; ++i) {
    if (i == 0 || mode == NM_ADJ_PAIR || std::fabs(lam[i] - lam[i - 1]) > tol * std::fabs(lam[i - 1])) ++ng;
    grp[i] = ng - 1;
  }
  if (mode == NM_ADJ_MULTIPLET) {
    std::fill(grad, grad + (size_t)ng * ntet * 3, 0.0);
    for (int i = 0; i < k; ++i) {
      const double* src = pair.data() + (size_t)i * ntet * 3;
      double* dst = grad + (size_t)grp[i] * ntet * 3;
      for (size_t q = 0; q < (size_t)ntet * 3; ++q) dst[q] += src[q];
    }
  }
  if (group) std::copy(grp.begin(), grp.end(), group);
  if (ngroups) *ngroups = ng;
  return NM_OK;
}
