"""CPU model of the integer-digit Gram's number format (the mixed-precision QGT contraction).

The tcgen05 Gram (quantum_geometric_tensor_gb300/csrc/cuda/qgt_gram_digits.cu) writes every complex64
amplitude of row r as x = u_r (D + l1 + l2): u_r = 2^(e_r - mbits) from the row maximum (rowmax <
2^e_r), D = rint(x / u_r) an integer held exactly in FP16, l1 = fp16(x / u_r - D), l2 = fp16(x / u_r -
D - l1).  Its D x D' products are accumulated by the FP32 tensor accumulator, which is exact only if
every partial sum stays an integer below 2^24; the kernel picks mbits so that a K range of kc
amplitudes obeys kc (M^2 + sqrt(2) M + 1/2) <= 2^23 (M = 2^mbits), and keeps the residual terms
D l1', l1 D', l1 l1', D l2', l2 D' in a second accumulator.  This test restates that format in numpy
and checks, on the rows the bound is tight for (every amplitude at the row maximum) and on random
rows:
- the digits stay within |D| <= M + 1 per part and the exact partial sums within 2^23;
- D + l1 + l2 reconstructs x / u to FP32 accuracy of the row maximum;
- the 12-term Gram (the terms the kernel keeps) equals the exact Gram of the complex64 rows to
  ~1e-7 relative, the size of error the digit Gram reaches on the GPU (1e-6 metric target)."""
import numpy as np
import pytest

F16 = np.float16


def mbits_for(kc):
    """The kernel's digit width for K ranges of kc amplitudes (qgt_dev_dg_gram_create)."""
    mb = 10
    while mb > 1:
        M = float(1 << mb)
        if kc * (M * M + 1.4143 * M + 0.5) <= 8388608.0:
            break
        mb -= 1
    return mb


def unit_exp(rowmax, mbits):
    """rowmax < 2^e; the row's unit is u = 2^(e - mbits) (unit_exp of the kernel)."""
    if not rowmax > 0:
        return 0
    _, e = np.frexp(np.float32(rowmax))
    return int(e) - mbits


def digits(x, mbits):
    """x: complex64 row -> (u, D, l1, l2) as float64 arrays of complex values (parts kept apart)."""
    rm = float(np.max(np.abs(x.astype(np.complex64))))
    iu = np.float32(np.ldexp(1.0, -unit_exp(rm, mbits)))
    out = []
    for part in (x.real.astype(np.float32), x.imag.astype(np.float32)):
        y = part * iu                                   # exact: a power of two
        d = np.rint(y).astype(np.float32)
        l = (y - d).astype(np.float32)
        l1 = l.astype(F16)
        l2 = (l - l1.astype(np.float32)).astype(F16)
        assert np.all(d.astype(F16).astype(np.float32) == d)   # D is exact in FP16
        out.append((d.astype(np.float64), l1.astype(np.float64), l2.astype(np.float64)))
    (dr, l1r, l2r), (di, l1i, l2i) = out
    return 1.0 / float(iu), dr + 1j * di, l1r + 1j * l1i, l2r + 1j * l2i


def gram12(a, b):
    """<a|b> from the kernel's 12 terms: D D' exactly, D l1' + l1 D' + l1 l1' + D l2' + l2 D'."""
    ua, Da, l1a, l2a = a
    ub, Db, l1b, l2b = b
    exact = np.vdot(Da, Db)
    rest = np.vdot(Da, l1b) + np.vdot(l1a, Db) + np.vdot(l1a, l1b) + np.vdot(Da, l2b) + np.vdot(l2a, Db)
    return ua * ub * (exact + rest), exact


@pytest.mark.parametrize("kc", [16, 64, 256, 1024])
def test_digit_width_bound(kc):
    """The chosen width keeps the exact accumulator below 2^23 even when every amplitude sits at
    the row maximum with both parts of the same size (the worst case of |Re D| + |Im D|)."""
    mb = mbits_for(kc)
    assert 1 <= mb <= 10 and (kc != 1024 or mb == 6)
    # rowmax just below 2^e: |x| / u just below M, parts up to M / sqrt(2) each, rounded outward
    x = np.full(kc, (1 - 2.0 ** -20) * np.exp(0.25j * np.pi), np.complex64)
    u, D, _, _ = digits(x, mb)
    M = 1 << mb
    assert np.all(np.abs(D.real) <= M + 1) and np.all(np.abs(D.imag) <= M + 1)
    s = np.vdot(D, D)
    partial = np.cumsum(np.conj(D) * D)
    assert abs(s.real) <= 2 ** 23 and np.all(np.abs(partial.real) <= 2 ** 23)
    # the same with opposite-phase rows (the largest off-diagonal sums)
    y = np.full(kc, (1 - 2.0 ** -20) * np.exp(-0.75j * np.pi), np.complex64)
    _, Dy, _, _ = digits(y, mb)
    cross = np.cumsum(np.conj(D) * Dy)
    assert np.all(np.abs(cross.real) <= 2 ** 23) and np.all(np.abs(cross.imag) <= 2 ** 23)


def test_reconstruction_and_gram_accuracy():
    rng = np.random.default_rng(7)
    kc = 1024
    mb = mbits_for(kc)
    rows = []
    for k in range(12):
        # derivative-state-like rows: a few large amplitudes over a wide spread of small ones
        amp = rng.standard_normal(kc) * np.exp(rng.uniform(-8, 0, kc))
        z = (amp * np.exp(1j * rng.uniform(0, 2 * np.pi, kc))).astype(np.complex64)
        rows.append(z)
    dig = [digits(z, mb) for z in rows]
    for z, (u, D, l1, l2) in zip(rows, dig):
        rec = u * (D + l1 + l2)
        rm = np.max(np.abs(z))
        assert np.max(np.abs(rec - z.astype(np.complex128))) <= 2.0 ** -22 * rm
    G = np.array([[np.vdot(a.astype(np.complex128), b.astype(np.complex128)) for b in rows] for a in rows])
    G12 = np.zeros_like(G)
    for i, a in enumerate(dig):
        for j, b in enumerate(dig):
            G12[i, j], exact = gram12(a, b)
            assert exact.real == np.round(exact.real) and exact.imag == np.round(exact.imag)
    err = np.abs(G12 - G).max() / np.abs(G).max()
    assert err < 2e-7, err
