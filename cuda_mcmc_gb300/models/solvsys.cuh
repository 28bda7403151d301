// solvsys.cuh -- the two-equation system of the reference's solvsys example
// (examples/solvsys/model.cuh:51-54) as a model.cuh plugin:
//   datum 0:  x^P1 + y^P2      (coor[0] = P1, coor[1] = P2)
//   datum 1:  -K x + y         (coor[2] = K)
__device__ int model(CCalcModel *mc, int id, int ipt, int imd, int ipass)
{
  const float x = mc->pcur[ipt], y = mc->pcur[ipt + 1];
  if (id == 0)
    mc->datm[imd] = powf(x, mc->coor[0]) + powf(y, mc->coor[1]);
  else
    mc->datm[imd] = -mc->coor[2] * x + y;
  return 1;
}
