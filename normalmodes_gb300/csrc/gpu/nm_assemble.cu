// Element-level assembly of the JOB = 1 operators on the GPU: the element
// matrices of CGE3D_ISO / CGFSE3D_ISO without gravity
// (src/mod_cg_create_matrix.f90:103-1266) computed per tetrahedron and added
// into given CSR structures (:1269-2033), the same formulas and element
// classification as the host assembly (nm_model.cpp):
//   * geometry: invJ = 2 B^-1, detJ = det B / 8 with B the edge matrix from
//     vertex 1 (src/mod_geometry.f90:2216-2240, :1401-1407); face normals
//     and sJac = |cross| / 4 (:2265-2304, :1418-1428);
//   * solid element (max mu >= 1e-8 or a solid-only model): lambda and mu
//     weighted reference mass, symmetrised; the 3x3 operator blocks
//     (OP_ij) times detJ into A (solid model) or Ad; the mass rho M detJ
//     (solid model: (rho_a M_ab + M_ab rho_b) / 2; general model: mean rho)
//     into B (:980-1266, :279-452);
//   * fluid element: the coupling O_i = (M D_i + (D_i^T M)^T) / 2 detJ into E
//     and ET, -detJ diag(kappa^-1/2) M diag(kappa^-1/2) into Ap, mean rho
//     M detJ into B (:453-640);
//   * fluid-solid interface face (three vertices with 6 DOFs): the face
//     coupling -n sJac MassF into ET and E (:803-953).
// One thread per element; the element's blocks live in local memory and are
// added with double atomics at positions found by binary search in the CSR
// rows (column lists sorted, as the reference's structure builder leaves
// them), so the sums are the host's up to the order of the additions.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "nm_internal.h"

namespace nmg {
namespace {

struct DevCsr {
  const int* rp;
  const int* ci;
  double* v;
};

__device__ __forceinline__ int dfind(const DevCsr& C, int row, int col) {
  int lo = C.rp[row], hi = C.rp[row + 1];
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (C.ci[mid] < col) lo = mid + 1;
    else hi = mid;
  }
  return (lo < C.rp[row + 1] && C.ci[lo] == col) ? lo : -1;
}

__device__ __forceinline__ void add(const DevCsr& C, int pos, double x, int* status) {
  if (pos < 0) {
    atomicExch(status, 1);  // structure miss: the caller's CSR lacks an entry
    return;
  }
  atomicAdd(&C.v[pos], x);
}

struct AsmArgs {
  int ntet, general;
  const int *tets, *vstt, *rnum, *pstt;
  const double *xyz, *vp, *vs, *rho, *M, *D, *MF;
  const int* FM;
  DevCsr A, B, Ap, E, ET;
  int* status;
};

// C = A B for P x P row-major matrices, sums in k order (as the host's mm)
template <int P>
__device__ __forceinline__ void mmP(const double* A, const double* B, double* C) {
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j) {
      double s = 0.0;
      for (int k = 0; k < P; ++k) s += A[i * P + k] * B[k * P + j];
      C[i * P + j] = s;
    }
}
// C = A^T B
template <int P>
__device__ __forceinline__ void mtP(const double* A, const double* B, double* C) {
  for (int i = 0; i < P; ++i)
    for (int j = 0; j < P; ++j) {
      double s = 0.0;
      for (int k = 0; k < P; ++k) s += A[k * P + i] * B[k * P + j];
      C[i * P + j] = s;
    }
}

template <int P>
__global__ void __launch_bounds__(128) k_assemble(AsmArgs a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.ntet) return;
  constexpr int NF = P == 4 ? 3 : 6;  // nodes per face
  const int vord[4] = {0, P == 4 ? 1 : 2, P == 4 ? 2 : 5, P == 4 ? 3 : 9};
  const int* nodes = a.tets + (size_t)P * k;
  // ---- geometry
  double v[4][3];
  for (int i = 0; i < 4; ++i)
    for (int c = 0; c < 3; ++c) v[i][c] = a.xyz[3 * (size_t)nodes[vord[i]] + c];
  double Bm[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) Bm[r][c] = v[r + 1][c] - v[0][c];
  const double det = Bm[0][0] * (Bm[1][1] * Bm[2][2] - Bm[1][2] * Bm[2][1]) -
                     Bm[0][1] * (Bm[1][0] * Bm[2][2] - Bm[1][2] * Bm[2][0]) +
                     Bm[0][2] * (Bm[1][0] * Bm[2][1] - Bm[1][1] * Bm[2][0]);
  if (det == 0.0) {
    atomicExch(a.status, 2);
    return;
  }
  double invJ[3][3];
  invJ[0][0] = (Bm[1][1] * Bm[2][2] - Bm[1][2] * Bm[2][1]) / det;
  invJ[0][1] = (Bm[0][2] * Bm[2][1] - Bm[0][1] * Bm[2][2]) / det;
  invJ[0][2] = (Bm[0][1] * Bm[1][2] - Bm[0][2] * Bm[1][1]) / det;
  invJ[1][0] = (Bm[1][2] * Bm[2][0] - Bm[1][0] * Bm[2][2]) / det;
  invJ[1][1] = (Bm[0][0] * Bm[2][2] - Bm[0][2] * Bm[2][0]) / det;
  invJ[1][2] = (Bm[0][2] * Bm[1][0] - Bm[0][0] * Bm[1][2]) / det;
  invJ[2][0] = (Bm[1][0] * Bm[2][1] - Bm[1][1] * Bm[2][0]) / det;
  invJ[2][1] = (Bm[0][1] * Bm[2][0] - Bm[0][0] * Bm[2][1]) / det;
  invJ[2][2] = (Bm[0][0] * Bm[1][1] - Bm[0][1] * Bm[1][0]) / det;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) invJ[r][c] *= 2.0;
  const double detJ = det / 8.0;
  // ---- material
  double lam[P], mu[P], rhot[P];
  double maxmu = 0.0, srho = 0.0;
  for (int l = 0; l < P; ++l) {
    const size_t q = (size_t)P * k + l;
    const double c44 = a.rho[q] * a.vs[q] * a.vs[q];
    const double c33 = a.rho[q] * a.vp[q] * a.vp[q] - 2 * c44;
    lam[l] = c33;
    mu[l] = c44;
    rhot[l] = a.rho[q];
    maxmu = fmax(maxmu, c44);
    srho += rhot[l];
  }
  const bool solid = !a.general || maxmu >= 1e-8;
  double D[3][P * P];
  for (int i = 0; i < 3; ++i)
    for (int e = 0; e < P * P; ++e)
      D[i][e] = invJ[i][0] * a.D[e] + invJ[i][1] * a.D[P * P + e] + invJ[i][2] * a.D[2 * P * P + e];
  double Mrho[P * P];
  if (solid && !a.general) {
    for (int p = 0; p < P; ++p)
      for (int q = 0; q < P; ++q)
        Mrho[p * P + q] = (rhot[p] * a.M[p * P + q] + a.M[p * P + q] * rhot[q]) / 2.0;
  } else {
    for (int e = 0; e < P * P; ++e) Mrho[e] = a.M[e] * srho / (double)P;
  }
  if (solid) {
    double Ml[P * P], Mm[P * P];
    for (int p = 0; p < P; ++p)
      for (int q = 0; q < P; ++q) {
        Ml[p * P + q] = a.M[p * P + q] * lam[q];
        Mm[p * P + q] = a.M[p * P + q] * mu[q];
      }
    for (int p = 0; p < P; ++p)
      for (int q = p; q < P; ++q) {
        const double l1 = (Ml[p * P + q] + Ml[q * P + p]) / 2.0, m1 = (Mm[p * P + q] + Mm[q * P + p]) / 2.0;
        Ml[p * P + q] = Ml[q * P + p] = l1;
        Mm[p * P + q] = Mm[q * P + p] = m1;
      }
    double OP1[3][P * P], OP2[3][P * P], OPt[3][P * P], OPs[P * P];
    for (int e = 0; e < P * P; ++e) OPs[e] = 0.0;
    for (int i = 0; i < 3; ++i) {
      mmP<P>(Ml, D[i], OP1[i]);
      mmP<P>(Mm, D[i], OP2[i]);
      mtP<P>(D[i], OP2[i], OPt[i]);
      for (int e = 0; e < P * P; ++e) OPs[e] += OPt[i][e];
    }
    const DevCsr& Am = a.A;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double OPij[P * P];
        if (i == j) {
          double tmp[P * P];
          mtP<P>(D[i], OP1[i], tmp);
          for (int e = 0; e < P * P; ++e) tmp[e] = OPs[e] + OPt[i][e] + tmp[e];
          for (int p = 0; p < P; ++p)
            for (int q = 0; q < P; ++q) OPij[p * P + q] = (tmp[p * P + q] + tmp[q * P + p]) / 2.0;
        } else {
          double a1[P * P], a2[P * P], b1[P * P], b2[P * P];
          mtP<P>(D[i], OP1[j], a1);
          mtP<P>(D[j], OP2[i], a2);
          mtP<P>(D[j], OP1[i], b1);
          mtP<P>(D[i], OP2[j], b2);
          for (int p = 0; p < P; ++p)
            for (int q = 0; q < P; ++q)
              OPij[p * P + q] = ((b1[q * P + p] + b2[q * P + p]) + (a1[p * P + q] + a2[p * P + q])) / 2.0;
        }
        for (int p = 0; p < P; ++p) {
          const int row = a.vstt[nodes[p]] + i;
          for (int q = 0; q < P; ++q) add(Am, dfind(Am, row, a.vstt[nodes[q]] + j), OPij[p * P + q] * detJ, a.status);
          if (i == j)
            for (int q = 0; q < P; ++q)
              add(a.B, dfind(a.B, row, a.vstt[nodes[q]] + i), Mrho[p * P + q] * detJ, a.status);
        }
      }
    return;
  }
  // ---- fluid element
  double lamiv[P];
  for (int l = 0; l < P; ++l) lamiv[l] = 1.0 / sqrt(lam[l]);
  for (int p = 0; p < P; ++p) {
    const int prow = a.pstt[nodes[p]];
    for (int q = 0; q < P; ++q)
      add(a.Ap, dfind(a.Ap, prow, a.pstt[nodes[q]]), -(detJ * ((lamiv[p] * a.M[p * P + q]) * lamiv[q])), a.status);
  }
  for (int i = 0; i < 3; ++i) {
    double G[P * P], Ot[P * P];
    mmP<P>(a.M, D[i], G);
    mtP<P>(D[i], a.M, Ot);
    for (int p = 0; p < P; ++p) {
      const int np_ = nodes[p];
      const int row = a.vstt[np_] + a.rnum[np_] - 3 + i;  // fluid copy of the displacement DOF
      const int prow = a.pstt[np_];
      for (int q = 0; q < P; ++q) {
        const int nq = nodes[q];
        const double opq = (G[p * P + q] + Ot[q * P + p]) / 2.0;  // O_i(p, q)
        const double oqp = (G[q * P + p] + Ot[p * P + q]) / 2.0;  // O_i(q, p)
        add(a.E, dfind(a.E, row, a.pstt[nq]), opq * detJ, a.status);
        add(a.ET, dfind(a.ET, prow, a.vstt[nq] + a.rnum[nq] - 3 + i), oqp * detJ, a.status);
        add(a.B, dfind(a.B, row, a.vstt[nq] + a.rnum[nq] - 3 + i), Mrho[p * P + q] * detJ, a.status);
      }
    }
  }
  // fluid-solid interface: the face opposite the one vertex without 6 DOFs
  int cout = 0, fcid = -1;
  for (int w = 0; w < 4; ++w) {
    if (a.rnum[nodes[vord[w]]] == 6) ++cout;
    else fcid = w;
  }
  if (cout != 3) return;
  // outward normal and sJac of face fcid (the other three vertices in order)
  const double* vr = v[fcid];
  const double* w3[3];
  int kk = 0;
  for (int j = 0; j < 4; ++j)
    if (j != fcid) w3[kk++] = v[j];
  double e1[3], e2[3], nn[3];
  for (int c = 0; c < 3; ++c) {
    e1[c] = w3[1][c] - w3[0][c];
    e2[c] = w3[2][c] - w3[0][c];
  }
  nn[0] = e1[1] * e2[2] - e1[2] * e2[1];
  nn[1] = e1[2] * e2[0] - e1[0] * e2[2];
  nn[2] = e1[0] * e2[1] - e1[1] * e2[0];
  const double sj = sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
  for (int c = 0; c < 3; ++c) nn[c] /= sj;
  double dot = 0.0;
  for (int c = 0; c < 3; ++c) dot += (vr[c] - w3[0][c]) * nn[c];
  if (dot > 0)
    for (int c = 0; c < 3; ++c) nn[c] = -nn[c];
  const double sJac = sj / 4.0;
  const int* Fm = a.FM + NF * fcid;
  const double* MF = a.MF + (size_t)NF * NF * fcid;
  for (int p = 0; p < NF; ++p) {
    const int np_ = nodes[Fm[p]];
    const int prow = a.pstt[np_];
    for (int q = 0; q < NF; ++q) {
      const int nq = nodes[Fm[q]];
      const int pos = dfind(a.ET, prow, a.vstt[nq]);
      for (int c = 0; c < 3; ++c) add(a.ET, pos < 0 ? -1 : pos + c, -(nn[c] * sJac * MF[q * NF + p]), a.status);
    }
    for (int c = 0; c < 3; ++c) {
      const int row = a.vstt[np_] + c;
      for (int q = 0; q < NF; ++q)
        add(a.E, dfind(a.E, row, a.pstt[nodes[Fm[q]]]), -(nn[c] * sJac * MF[p * NF + q]), a.status);
    }
  }
}

template <typename T>
int upload(const T* h, size_t n, T** d) {
  if (cudaMalloc(d, sizeof(T) * std::max<size_t>(n, 1)) != cudaSuccess) return NM_ERR_OOM;
  if (n && cudaMemcpy(*d, h, sizeof(T) * n, cudaMemcpyHostToDevice) != cudaSuccess) return NM_ERR_CUDA;
  return NM_OK;
}

}  // namespace
}  // namespace nmg

using namespace nmg;

extern "C" int nm_assemble(const nm_elem_model* em, nm_csr_fill* A, nm_csr_fill* B, nm_csr_fill* Ap,
                           nm_csr_fill* E, nm_csr_fill* ET, double* seconds) {
  if (!em || !A || !B || (em->pnp != 4 && em->pnp != 10) || em->ntet <= 0) return NM_ERR_ARG;
  if (em->g0) return NM_ERR_ARG;  // the reference-gravity terms are assembled on the host
  const bool general = em->fluid_solid != 0;
  if (general && (!Ap || !E || !ET)) return NM_ERR_ARG;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    return NM_ERR_CUDA;
  }
  const int p = em->pnp, nf = p == 4 ? 3 : 6;
  const size_t nt = (size_t)em->ntet;
  std::vector<void*> owned;
  auto cleanup = [&]() {
    for (void* q : owned) cudaFree(q);
    owned.clear();
  };
  int rc = NM_OK;
  auto up = [&](const auto* h, size_t n, auto** d) {
    if (rc) return;
    rc = upload(h, n, d);
    owned.push_back((void*)*d);
  };
  AsmArgs a{};
  a.ntet = em->ntet;
  a.general = general;
  int *dt = nullptr, *dvstt = nullptr, *drnum = nullptr, *dpstt = nullptr, *dfm = nullptr;
  double *dxyz = nullptr, *dvp = nullptr, *dvs = nullptr, *drho = nullptr, *dM = nullptr, *dD = nullptr, *dMF = nullptr;
  up(em->tets, nt * p, &dt);
  up(em->xyz, 3 * (size_t)em->nnode, &dxyz);
  up(em->vstt, (size_t)em->nnode, &dvstt);
  up(em->rnum, (size_t)em->nnode, &drnum);
  up(em->pstt, (size_t)em->nnode, &dpstt);
  up(em->vp, nt * p, &dvp);
  up(em->vs, nt * p, &dvs);
  up(em->rho, nt * p, &drho);
  up(em->ref_mass, (size_t)p * p, &dM);
  up(em->ref_drst, 3 * (size_t)p * p, &dD);
  if (general) {
    if (!em->ref_massf || !em->ref_fmask) rc = rc ? rc : NM_ERR_ARG;
    else {
      up(em->ref_massf, 4 * (size_t)nf * nf, &dMF);
      up(em->ref_fmask, 4 * (size_t)nf, &dfm);
    }
  }
  a.tets = dt;
  a.xyz = dxyz;
  a.vstt = dvstt;
  a.rnum = drnum;
  a.pstt = dpstt;
  a.vp = dvp;
  a.vs = dvs;
  a.rho = drho;
  a.M = dM;
  a.D = dD;
  a.MF = dMF;
  a.FM = dfm;
  nm_csr_fill* outs[5] = {A, B, Ap, E, ET};
  DevCsr* dcs[5] = {&a.A, &a.B, &a.Ap, &a.E, &a.ET};
  for (int q = 0; q < 5 && !rc; ++q) {
    if (!outs[q]) continue;
    const nm_csr_fill* o = outs[q];
    const size_t nnz = (size_t)o->rowptr[o->nrows];
    int *rp = nullptr, *ci = nullptr;
    double* v = nullptr;
    up(o->rowptr, (size_t)o->nrows + 1, &rp);
    up(o->col, nnz, &ci);
    if (!rc && cudaMalloc(&v, sizeof(double) * std::max<size_t>(nnz, 1)) != cudaSuccess) rc = NM_ERR_OOM;
    if (!rc) {
      owned.push_back(v);
      cudaMemset(v, 0, sizeof(double) * nnz);
    }
    dcs[q]->rp = rp;
    dcs[q]->ci = ci;
    dcs[q]->v = v;
  }
  int* dstatus = nullptr;
  if (!rc && cudaMalloc(&dstatus, sizeof(int)) != cudaSuccess) rc = NM_ERR_OOM;
  if (rc) {
    cudaFree(dstatus);
    cleanup();
    return rc;
  }
  cudaMemset(dstatus, 0, sizeof(int));
  a.status = dstatus;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0);
  const int thr = 128, grid = (int)((nt + thr - 1) / thr);
  if (p == 4) k_assemble<4><<<grid, thr>>>(a);
  else k_assemble<10><<<grid, thr>>>(a);
  add_launches(1);
  cudaEventRecord(e1);
  int st = 0;
  cudaError_t ce = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (seconds) *seconds = 1e-3 * ms;
  if (ce == cudaSuccess) ce = cudaMemcpy(&st, dstatus, sizeof(int), cudaMemcpyDeviceToHost);
  if (ce == cudaSuccess)
    for (int q = 0; q < 5; ++q)
      if (outs[q] && ce == cudaSuccess)
        ce = cudaMemcpy(outs[q]->val, dcs[q]->v, sizeof(double) * (size_t)outs[q]->rowptr[outs[q]->nrows],
                        cudaMemcpyDeviceToHost);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(dstatus);
  cleanup();
  if (ce != cudaSuccess) return NM_ERR_CUDA;
  if (st == 2) return NM_ERR_NUMERIC;  // flat tetrahedron
  if (st == 1) return NM_ERR_ARG;      // the CSR structure lacks an entry the element needs
  return NM_OK;
}
