// nlsys.cuh -- an n-equation nonlinear system as a model.cuh plugin:
//   datum k:  sum_j A_kj sin(x_j) + B_kj x_j^2      (compared with dat[k] = b_k)
// with coor = [A | B], A and B each [ndat][nptot] row-major.
__device__ int model(CCalcModel *mc, int id, int ipt, int imd, int ipass)
{
  const int n = mc->nptot;
  const float *x = mc->pcur + ipt;
  const float *A = mc->coor + id * n;
  const float *B = mc->coor + mc->ndat * n + id * n;
  float s = 0.0f;
  for (int j = 0; j < n; ++j) s += A[j] * sinf(x[j]) + B[j] * x[j] * x[j];
  mc->datm[imd] = s;
  return 1;
}
