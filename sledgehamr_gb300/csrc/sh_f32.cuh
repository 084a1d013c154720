/* Explicitly rounded FP32 arithmetic shared by the FP32 stage kernels of
 * ensembles (sh_fast.cu, sh_fast_tma.cuh) and of FP32 levels
 * (sh_stage32.cuh). */
#ifndef SH_F32_CUH_
#define SH_F32_CUH_

namespace sh {

/* FP32 arithmetic of the axion stage kernels with every operation rounded
 * on its own (no contraction into fused multiply-adds), so that the
 * register-pipelined and the tensor-copy kernels, which share these
 * functions, give bit-identical results whatever the compiler fuses in its
 * surroundings. */
namespace f32 {
__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
/* stage position y + cm y' + ck K */
__device__ __forceinline__ float stage_pos(float y, float m, float k, float cm, float ck) {
    return add(y, add(mul(cm, m), mul(ck, k)));
}
/* 7-point Laplacian from the centre and the six neighbours (x+, x-, y+,
 * y-, z+, z-) */
__device__ __forceinline__ float lap7(float c, float xp, float xm, float yp, float ym, float zp,
                                      float zm, float inv_dx2) {
    float s = add(xp, xm);
    s = add(s, add(yp, ym));
    s = add(s, add(zp, zm));
    return mul(sub(s, mul(6.f, c)), inv_dx2);
}
/* 13-point Laplacian: s1 and s2 the sums of the first and second rings */
__device__ __forceinline__ float lap13(float c, float s1, float s2, float inv12dx2) {
    return mul(sub(sub(mul(16.f, s1), s2), mul(90.f, c)), inv12dx2);
}
/* sum of a ring: (x+, x-), (y+, y-), (z+, z-) */
__device__ __forceinline__ float ring(float xp, float xm, float yp, float ym, float zp,
                                      float zm) {
    float s = add(xp, xm);
    s = add(s, add(yp, ym));
    return add(s, add(zp, zm));
}
/* lambda (eta^2 (|Psi|^2 - 1) + c) */
__device__ __forceinline__ float potential(float p0, float p1, float lam, float eta2, float cst) {
    return mul(lam, add(mul(eta2, sub(add(mul(p0, p0), mul(p1, p1)), 1.f)), cst));
}
/* friction Pi + lap - Psi v */
__device__ __forceinline__ float accel(float q, float lap, float p, float v, float friction) {
    return sub(add(mul(friction, q), lap), mul(p, v));
}
/* RKN4 final increments: position h y0' + h^2 (K0/6 + K1/3), momentum
 * h ((K0 + K2)/6 + 2 K1/3) */
__device__ __forceinline__ float dpos(float q, float ka, float kb, float h, float h2) {
    return add(mul(h, q), mul(h2, add(mul(ka, 1.f / 6.f), mul(kb, 1.f / 3.f))));
}
__device__ __forceinline__ float dmom(float ka, float kb, float k, float h) {
    return mul(h, add(mul(add(ka, k), 1.f / 6.f), mul(kb, 2.f / 3.f)));
}
/* compensated y += d (c holds minus the lost low part) */
__device__ __forceinline__ void kahan(float &y, float d, float &c) {
    const float v = sub(d, c);
    const float t = add(y, v);
    c = sub(sub(t, y), v);
    y = t;
}
} // namespace f32

} // namespace sh

#endif
