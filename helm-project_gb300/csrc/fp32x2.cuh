// Packed-pair FP32 arithmetic (f32x2) and the compensated accumulation
// steps shared by the split-FP32 apply kernels.
#pragma once

namespace axgb {

struct F2 {
    unsigned long long v;
};
__device__ __forceinline__ F2 pk(float a, float b) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(F2 r, float &a, float &b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r.v)); }
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}

// One compensated step for one field: s + c accumulates (hi + lo) * x.
// TwoSum of s and p = fl(h*x) gives t and the error (s - a) + (p - b), with
// b = t - s and a = t - b. The second part is formed together with the
// product error as fma(h, x, -b) = fl(h*x - b): one rounding at the scale
// of the error term instead of a separate exact product error. Here
// bn = s - t is -b exactly (rounding is sign-symmetric), so a = t + bn. The
// low weight enters as c = fma(lo, x, c), then c += e. Nine operations.
__device__ __forceinline__ void csum1(float &s, float &c, float h, float l, float x) {
    const float p = __fmul_rn(h, x);
    const float t = __fadd_rn(s, p);
    const float bn = __fsub_rn(s, t);
    const float a = __fadd_rn(t, bn);
    const float e = __fadd_rn(__fsub_rn(s, a), __fmaf_rn(h, x, bn));
    c = __fadd_rn(__fmaf_rn(l, x, c), e);
    s = t;
}

// The same step for two fields at once (each half bitwise csum1). The two
// products are formed by scalar multiplies with explicit rounding: a packed
// multiply whose only use is the next packed add gets fused with it into
// one packed fma by the code generator (t = fl(s + h*x) instead of
// fl(s + fl(h*x))), which breaks the error-free sum.
__device__ __forceinline__ void csum2(F2 &s, F2 &c, float h, F2 hp, F2 lp, float xa, float xb) {
    const F2 x = pk(xa, xb);
    const F2 p = pk(__fmul_rn(h, xa), __fmul_rn(h, xb));
    const F2 t = add2(s, p);
    const F2 bn = sub2(s, t);
    const F2 a = add2(t, bn);
    const F2 e = add2(sub2(s, a), fma2(hp, x, bn));
    c = add2(fma2(lp, x, c), e);
    s = t;
}

// The same step with the compensation carried negated (cn = -c, ln = -lo):
// fma(-lo, x, -c) = -fma(lo, x, c) and -c - e = -(c + e) exactly, so the row
// value s - cn is bitwise that of csum1.
__device__ __forceinline__ void cstepn(F2 &s, F2 &cn, float h, F2 hp, F2 ln, float xa, float xb) {
    const F2 x = pk(xa, xb);
    const F2 p = pk(__fmul_rn(h, xa), __fmul_rn(h, xb));  // not fusable (see csum2)
    const F2 t = add2(s, p);
    const F2 bn = sub2(s, t);
    const F2 a = add2(t, bn);
    const F2 e = add2(sub2(s, a), fma2(hp, x, bn));
    cn = sub2(fma2(ln, x, cn), e);
    s = t;
}

// The cstepn step for two rows side by side (one field each): w = (hi_a,
// hi_b, -lo_a, -lo_b); each half is bitwise csum1 of its own row.
__device__ __forceinline__ void cstep_pair(F2 &s, F2 &cn, float4 w, float xa, float xb) {
    const F2 x = pk(xa, xb);
    const F2 p = pk(__fmul_rn(w.x, xa), __fmul_rn(w.y, xb));  // not fusable (see csum2)
    const F2 t = add2(s, p);
    const F2 bn = sub2(s, t);
    const F2 a = add2(t, bn);
    const F2 e = add2(sub2(s, a), fma2(pk(w.x, w.y), x, bn));
    cn = sub2(fma2(pk(w.z, w.w), x, cn), e);
    s = t;
}

// Low part of a row value. The stored value is r = fl(s + c); the exact
// rounding error of that sum (Knuth's TwoSum, exact for any operand order)
// is returned, so r + lo represents s + c to within FP32 round-off of c's
// own error term. Used by the hi+lo output form of the split apply.
__device__ __forceinline__ float sum_err(float s, float c, float r) {
    const float bp = __fsub_rn(r, s);
    const float ap = __fsub_rn(r, bp);
    return __fadd_rn(__fsub_rn(s, ap), __fsub_rn(c, bp));
}

// ─── rows longer than 32 entries ──────────────────────────────────────────
// Order for a row of n > 32 entries: leaf j (j = 0..31) sums entries j,
// j+32, j+64, ... in order with csum1; the 32 leaves are combined by an
// in-order pairwise tree (leaves 2m and 2m+1 first, and so on) with
// lcombine; the row value is s + c of the root. Computed with lane = leaf
// and a shuffle butterfly over lane offsets 1, 2, ..., 16: every lane ends
// with the root, since TwoSum's error is exact in either operand order and
// the other additions are commutative. Rows of at most 32 entries are
// summed in entry order.
__device__ __forceinline__ void lcombine(float &s, float &c, float s2, float c2) {
    const float t = __fadd_rn(s, s2);
    const float bp = __fsub_rn(t, s);
    const float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(s2, bp));
    c = __fadd_rn(__fadd_rn(c, c2), e);
    s = t;
}

}  // namespace axgb
