// weno5_core.cuh -- the WENO5-JS directional derivative of weno5.h:1-70, as a
// device function templated on the arithmetic type.
#pragma once

namespace fmf {

__device__ __forceinline__ double absr(double x) { return fabs(x); }
__device__ __forceinline__ float absr(float x) { return fabsf(x); }

// Product-form weights: am1=(s2 s3)^2, am2=6(s1 s3)^2, am3=3(s1 s2)^2 and the
// mirrored ap*, evaluated in the reference's operation order.
template <class R>
__device__ __forceinline__ R weno5_dir(R vel00, R dfm5, R dfm3, R dfm1, R dfp1, R dfp3, R dfp5) {
  const R verysmall = (R)1.0e-80, d1_12 = (R)1.0 / (R)12.0;
  const R dfm_1 = dfm5 * (R)2.0 - dfm3 * (R)7.0 + dfm1 * (R)11.0;
  const R dfm_2 = -dfm3 + dfm1 * (R)5.0 + dfp1 * (R)2.0;
  const R dfm_3 = dfm1 * (R)2.0 + dfp1 * (R)5.0 - dfp3;
  const R dfp_1 = dfp5 * (R)2.0 - dfp3 * (R)7.0 + dfp1 * (R)11.0;
  const R dfp_2 = -dfp3 + dfp1 * (R)5.0 + dfm1 * (R)2.0;
  const R dfp_3 = dfp1 * (R)2.0 + dfm1 * (R)5.0 - dfm3;
  R t1, t2;
  t1 = dfm5 - dfm3 * (R)2.0 + dfm1; t2 = dfm5 - dfm3 * (R)4.0 + dfm1 * (R)3.0;
  const R sm_1 = (t1 * t1) * (R)13.0 + (t2 * t2) * (R)3.0;
  t1 = dfm3 - dfm1 * (R)2.0 + dfp1; t2 = dfm3 - dfp1;
  const R sm_2 = (t1 * t1) * (R)13.0 + (t2 * t2) * (R)3.0;
  t1 = dfm1 - dfp1 * (R)2.0 + dfp3; t2 = dfm1 * (R)3.0 - dfp1 * (R)4.0 + dfp3;
  const R sm_3 = (t1 * t1) * (R)13.0 + (t2 * t2) * (R)3.0;
  t1 = dfp5 - dfp3 * (R)2.0 + dfp1; t2 = dfp5 - dfp3 * (R)4.0 + dfp1 * (R)3.0;
  const R sp_1 = (t1 * t1) * (R)13.0 + (t2 * t2) * (R)3.0;
  t1 = dfp3 - dfp1 * (R)2.0 + dfm1; t2 = dfp3 - dfm1;
  const R sp_2 = (t1 * t1) * (R)13.0 + (t2 * t2) * (R)3.0;
  t1 = dfp1 - dfm1 * (R)2.0 + dfm3; t2 = dfp1 * (R)3.0 - dfm1 * (R)4.0 + dfm3;
  const R sp_3 = (t1 * t1) * (R)13.0 + (t2 * t2) * (R)3.0;
  R am_1 = sm_2 * sm_3, am_2 = sm_1 * sm_3, am_3 = sm_1 * sm_2;
  R ap_1 = sp_2 * sp_3, ap_2 = sp_1 * sp_3, ap_3 = sp_1 * sp_2;
  am_1 = am_1 * am_1;
  am_2 = am_2 * am_2;
  am_3 = am_3 * am_3;
  ap_1 = ap_1 * ap_1;
  ap_2 = ap_2 * ap_2;
  ap_3 = ap_3 * ap_3;
  am_2 = am_2 * (R)6.0;
  am_3 = am_3 * (R)3.0;
  ap_2 = ap_2 * (R)6.0;
  ap_3 = ap_3 * (R)3.0;
  const R dam = (R)1.0 / (am_1 + am_2 + am_3 + verysmall);
  const R dap = (R)1.0 / (ap_1 + ap_2 + ap_3 + verysmall);
  const R wgm_1 = am_1 * dam, wgm_3 = am_3 * dam;
  const R wgp_1 = ap_1 * dap, wgp_3 = ap_3 * dap;
  const R wgm_2 = (R)1.0 - wgm_1 - wgm_3;
  const R wgp_2 = (R)1.0 - wgp_1 - wgp_3;
  const R velab = absr(vel00);
  const R velm1 = vel00 + velab, velp1 = vel00 - velab;
  return (velm1 * (wgm_1 * dfm_1 + wgm_2 * dfm_2 + wgm_3 * dfm_3) +
          velp1 * (wgp_1 * dfp_1 + wgp_2 * dfp_2 + wgp_3 * dfp_3)) *
         d1_12;
}

// derivative along stride S at flat index c of field q
template <class R, class T>
__device__ __forceinline__ R weno5_line(const T* q, long c, long S, R vel) {
  const R m3 = (R)q[c - 3 * S], m2 = (R)q[c - 2 * S], m1 = (R)q[c - S], z0 = (R)q[c], p1 = (R)q[c + S],
          p2 = (R)q[c + 2 * S], p3 = (R)q[c + 3 * S];
  return weno5_dir<R>(vel, -m3 + m2, -m2 + m1, -m1 + z0, -z0 + p1, -p1 + p2, -p2 + p3);
}

}  // namespace fmf
