// rosenbrock.cuh -- N-dimensional Rosenbrock function as a model.cuh plugin.
//
// Follows the convention of the reference's Rosenbrock example
// (examples/search_Rosenbrock/model.cuh:40-41): datum 0 holds the function
// value, compared with dat[0] = 0, so chi^2 = f(x)^2.  With nptot = N,
//   f(x) = sum_{i=0}^{N-2} 100 (x_{i+1} - x_i^2)^2 + (1 - x_i)^2,
// which for N = 2 is the reference's (1 - x)^2 + 100 (y - x^2)^2.
__device__ int model(CCalcModel *mc, int id, int ipt, int imd, int ipass)
{
  if (id == 0) {
    const float *x = mc->pcur + ipt;
    float f = 0.0f;
    for (int i = 0; i + 1 < mc->nptot; ++i) {
      const float a = x[i + 1] - x[i] * x[i], b = 1.0f - x[i];
      f += 100.0f * a * a + b * b;
    }
    mc->datm[imd] = f;
  }
  return 1;
}
