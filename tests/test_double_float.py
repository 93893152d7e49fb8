"""The double-float product of the mixed forms' outer CG (k_spmv_df64,
k_spmv_rows_df64, k_spmm_df64): a host restatement of its arithmetic in
numpy float32 checks the accuracy the kernels rely on.

A = A_hi + A_lo and d = d_hi + d_lo as float pairs (hi = fl32(x), lo =
fl32(x - hi)); each product is the exact FP32 product of the high parts
(error recovered with a fused multiply-add) plus the two cross terms; the
sum is an unnormalised (sum, error) float pair updated with Knuth's two-sum.
The row sums must agree with FP64 to about 2^-44 of sum |a d| -- far below
the 1e-10 tolerance of the outer CG and far above plain FP32 (2^-24).
"""
import numpy as np

f32 = np.float32


def split(x):
    hi = x.astype(f32)
    lo = (x - hi.astype(np.float64)).astype(f32)
    return hi, lo


def fmaf(a, b, c):
    # a*b is exact in float64 for float32 inputs; one rounding to float32
    # after the float64 sum (the double rounding is far below the bound)
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def df_fma(sh, sl, ah, al, dh, dl):
    p = (ah * dh).astype(f32)
    pe = fmaf(ah, dh, -p)
    t = fmaf(ah, dl, fmaf(al, dh, pe))
    s = (sh + p).astype(f32)
    bb = (s - sh).astype(f32)
    e = ((sh - (s - bb)) + (p - bb)).astype(f32)
    return s, (sl + (e + t)).astype(f32)


def test_double_float_row_sums_reach_2_to_minus_44():
    rng = np.random.default_rng(11)
    nrow, nterm = 2000, 80          # 5 blocks x 16 columns per row of a Q3 operator
    # entries spanning several magnitudes with cancellation, as in LDG rows
    a = rng.standard_normal((nrow, nterm)) * np.exp(rng.uniform(-6, 6, (nrow, nterm)))
    d = rng.standard_normal((nrow, nterm))
    ah, al = split(a)
    dh, dl = split(d)
    sh = np.zeros(nrow, f32)
    sl = np.zeros(nrow, f32)
    for k in range(nterm):
        sh, sl = df_fma(sh, sl, ah[:, k], al[:, k], dh[:, k], dl[:, k])
    got = sh.astype(np.float64) + sl.astype(np.float64)
    ref = np.einsum("ij,ij->i", a, d)
    scale = np.einsum("ij,ij->i", np.abs(a), np.abs(d))
    rel = np.abs(got - ref) / scale
    assert rel.max() <= 2.0 ** -40, rel.max()
    assert np.median(rel) <= 2.0 ** -44, np.median(rel)
    # plain FP32 accumulation of fl32(a) fl32(d) for comparison: ~2^-24
    plain = np.zeros(nrow, f32)
    for k in range(nterm):
        plain = (plain + ah[:, k] * dh[:, k]).astype(f32)
    rel32 = np.abs(plain.astype(np.float64) - ref) / scale
    assert np.median(rel32) > 2.0 ** 12 * np.median(rel)
