"""The matrix form of Rotor::rotate that the split-precision ragged rotation
evaluates on the tensor cores, checked on the CPU against the oracle's
rotation (rotate_l, wignerd_collection.hpp:122-296; Rotor::rotate,
rotor.hpp:210-243).

Per rotated (n, l) vector v (complex coefficients after the real-to-complex
conversion and the gamma' phase), each X(+-pi/2) product is two real
matrices, one on the real parts and one on the imaginary parts:
  Re1[m][0] = D(m, 0),  Re1[m][m'] = 2 D(m, m') for m' >= 1 of the parity of l + m,
  Im1[m][m'] = 2 D(m, m') for m' >= 1 of the other parity,
with D(m, m') = (-1)^(m+m') d(m', m) for X(pi/2) and d(m', m) for X(-pi/2).
These are the tables the kernel slices (rot_table_kernel); the phases and the
conversions are applied where the operands are sliced and in the last pass."""
import numpy as np
import pytest

from oracle import zidx, zt_coeff_size


def wig_off(l):
    return l * (l + 1) * (2 * l + 1) // 6


def tables(wig, l, second):
    ld = l + 1
    d = wig[wig_off(l): wig_off(l) + ld * ld].reshape(ld, ld)  # d[m'][m]
    re = np.zeros((ld, ld))
    im = np.zeros((ld, ld))
    for m in range(ld):
        q = (l + m) & 1
        for mp in range(ld):
            D = d[mp, m] if (second or not ((m + mp) & 1)) else -d[mp, m]
            if mp == 0:
                re[m, 0] = D
            elif (mp & 1) == q:
                re[m, mp] = 2 * D
            else:
                im[m, mp] = 2 * D
    return re, im


def rotate_matrix_form(c, L, euler, wig, rtype):
    pi = np.pi
    if rtype == 0:
        a, b, g = euler[0] - 0.5 * pi, euler[1], euler[2] + 0.5 * pi
    else:
        a, b, g = -(euler[2] + 0.5 * pi), -euler[1], -(euler[0] - 0.5 * pi)
    out = c.copy()
    for l in range(L):
        re1, im1 = tables(wig, l, False)
        re2, im2 = tables(wig, l, True)
        m = np.arange(l + 1)
        for n in range(2 if l == 0 else l, L, 2):  # the rotated vectors
            base = zidx(n, l, 0)
            x = c[base: base + l + 1, 0] + 1j * c[base: base + l + 1, 1]
            x[1:] = (x[1:].real - 1j * x[1:].imag) / np.sqrt(2)
            v = x * np.exp(-1j * m * g)
            t = (re1 @ v.real + 1j * (im1 @ v.imag)) * np.exp(-1j * m * b)
            u = (re2 @ t.real + 1j * (im2 @ t.imag)) * np.exp(-1j * m * a)
            u[1:] = (u[1:].real - 1j * u[1:].imag) * np.sqrt(2)
            out[base: base + l + 1, 0] = u.real
            out[base: base + l + 1, 1] = u.imag
    return out


@pytest.mark.parametrize("L,rtype", [(1, 0), (2, 0), (9, 0), (16, 1), (23, 0)])
def test_matrix_form_equals_rotate(oracle, L, rtype):
    rng = np.random.default_rng(100 + L)
    c = rng.normal(size=(zt_coeff_size(L), 2))
    for n in range(L):
        for l in range(n & 1, n + 1, 2):
            c[zidx(n, l, 0), 1] = 0.0
    euler = rng.uniform(-3, 3, 3)
    want = oracle.zt_rotate(c.ravel().copy(), L, euler.copy(), rtype).reshape(-1, 2)
    got = rotate_matrix_form(c, L, euler, oracle.wignerd(L), rtype)
    assert np.max(np.abs(got - want)) <= 1e-14 * max(np.max(np.abs(want)), 1.0)
