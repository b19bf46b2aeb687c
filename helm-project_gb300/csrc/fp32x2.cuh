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
__device__ __forceinline__ void csum1(float &s, float &c, float h, float l, float x) {
    float p = __fmul_rn(h, x);
    float pe = __fmaf_rn(h, x, -p);
    float q = __fmaf_rn(l, x, pe);
    float t = __fadd_rn(s, p);
    float bp = __fsub_rn(t, s);
    float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(e, q));
}

// Same for two fields at once; hn = -hi (so mul gives -p exactly).
__device__ __forceinline__ void csum2(F2 &s, F2 &c, F2 h, F2 hn, F2 l, F2 x) {
    F2 pn = mul2(hn, x);
    F2 pe = fma2(h, x, pn);
    F2 q = fma2(l, x, pe);
    F2 t = sub2(s, pn);
    F2 bp = sub2(t, s);
    F2 a2 = sub2(s, sub2(t, bp));
    F2 a3 = add2(pn, bp);
    F2 e = sub2(a2, a3);
    s = t;
    c = add2(c, add2(e, q));
}

// Same arithmetic as csum2 (bitwise identical results) but without a
// negated-weight register pair: the product error is formed with -x and
// the compensation is carried negated (cn = -c); the row value is s - cn.
__device__ __forceinline__ void cstep2(F2 &s, F2 &cn, F2 h, F2 l, F2 x, F2 mone) {
    F2 nx = mul2(x, mone);
    F2 p = mul2(h, x);
    F2 pen = fma2(h, nx, p);  // p - h*x = -(product error), exact
    F2 t = add2(s, p);
    F2 bp = sub2(t, s);
    F2 a2 = sub2(s, sub2(t, bp));
    F2 a3 = sub2(p, bp);
    F2 e = add2(a2, a3);      // TwoSum error
    F2 u1 = fma2(l, nx, pen); // -(lo*x + product error)
    cn = add2(cn, sub2(u1, e));
    s = t;
}


// Bitwise negation of both halves on the integer pipe (keeps the FMA pipe
// for the arithmetic).
__device__ __forceinline__ F2 neg2(F2 a) {
    F2 r;
    r.v = a.v ^ 0x8000000080000000ull;
    return r;
}

// cstep2 with the negation on the integer pipe: 11 FMA-pipe operations per
// entry for two fields; results bitwise identical to csum1 on each field.
__device__ __forceinline__ void cstep2i(F2 &s, F2 &cn, F2 h, F2 l, F2 x) {
    F2 nx = neg2(x);
    F2 p = mul2(h, x);
    F2 pen = fma2(h, nx, p);
    F2 t = add2(s, p);
    F2 bp = sub2(t, s);
    F2 a2 = sub2(s, sub2(t, bp));
    F2 a3 = sub2(p, bp);
    F2 e = add2(a2, a3);
    F2 u1 = fma2(l, nx, pen);
    cn = add2(cn, sub2(u1, e));
    s = t;
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
