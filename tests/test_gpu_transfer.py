"""Unit parity of the two-level interface kernels with the transfer algebra.

Each production kernel of the interface (donor moments + prolongation +
donor populations, restriction, face fluxes, reflux) runs alone through
ak_refined_probe on states written into both levels, and is compared with
the oracle's restatement of refinement.py / interface.py applied to the same
states.  tests/test_transfer_algebra.py pins that restatement to the
reference's own NumPy outputs, so the chain reaches the reference.
"""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
O = pytest.importorskip("oracle.oracle")

POP_TOL = 1e-14  # absolute, zero-centred populations (FP64 on both sides)


@pytest.fixture(scope="module", autouse=True)
def _needs_device():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.fixture(scope="module")
def pair(golden):
    from tests.test_gpu_parity import refined_pair
    solver, oracle = refined_pair(golden["histories"]["refined_startup"])
    for _ in range(2):  # a developed, non-uniform state
        oracle.step()
    rng = np.random.default_rng(5)
    w = O.stencil()[1]
    coarse = oracle.coarse.interior().copy() + 2e-5 * w * (2 * rng.random(oracle.coarse.interior().shape) - 1)
    # the engine's fine block wraps z by index: the oracle's z padding dropped
    p = oracle.pad
    fine = oracle.fine.interior()[:, :, p:-p].copy()
    fine += 2e-5 * w * (2 * rng.random(fine.shape) - 1)
    yield solver, oracle, coarse, fine
    solver.close()


def load_states(solver, coarse, fine):
    from aerokinetic_gb300 import _native
    lib = solver._lib
    _native.check(lib.ak_set_pdf(solver._coarse, np.ascontiguousarray(coarse).ctypes.data_as(ctypes.c_void_p)))
    _native.check(lib.ak_set_pdf(solver._fine, np.ascontiguousarray(fine).ctypes.data_as(ctypes.c_void_p)))


def read(solver, level, shape):
    from aerokinetic_gb300 import _native
    out = np.empty(tuple(shape) + (27,))
    _native.check(solver._lib.ak_get_pdf(solver._coarse if level == 0 else solver._fine,
                                         out.ctypes.data_as(ctypes.c_void_p)))
    return out


def probe(solver, op, out=None):
    from aerokinetic_gb300 import _native
    n = ctypes.c_int64()
    ptr = out.ctypes.data_as(ctypes.c_void_p) if out is not None else None
    _native.check(solver._lib.ak_refined_probe(solver._handle, op, ptr, ctypes.byref(n)))
    return n.value


def z_padded(oracle, fine):
    p = oracle.pad
    return np.concatenate((fine[:, :, -p:], fine, fine[:, :, :p]), axis=2)


def test_donor_band_matches_the_prolongation(pair):
    solver, oracle, coarse, fine = pair
    load_states(solver, coarse, fine)
    probe(solver, 0)
    got = read(solver, 1, fine.shape[:3])
    block = oracle.donor_block(coarse)
    expected = oracle.fine_donors(block, block, 0.0)[:, :, oracle.pad:-oracle.pad]
    p = oracle.pad
    band = np.ones(fine.shape[:2], bool)
    band[p:-p, p:-p] = False
    assert band.sum() > 0
    np.testing.assert_allclose(got[band], expected[band], rtol=0, atol=POP_TOL)
    # the physical block is left as it was
    assert np.array_equal(got[~band], fine[~band])


def test_restriction_of_the_fine_block(pair):
    solver, oracle, coarse, fine = pair
    load_states(solver, coarse, fine)
    probe(solver, 1)
    got = read(solver, 0, coarse.shape[:3])
    p = oracle.pad
    expected = oracle.restrict(fine[p:-p, p:-p])
    np.testing.assert_allclose(got[oracle.box], expected, rtol=0, atol=POP_TOL)
    outside = np.ones(coarse.shape[:3], bool)
    outside[oracle.box] = False
    assert np.array_equal(got[outside], coarse[outside])


def test_face_flux_registers_and_reflux(pair):
    solver, oracle, coarse, fine = pair
    load_states(solver, coarse, fine)
    n = probe(solver, 2)
    regs = np.empty(n)
    probe(solver, 2, regs)
    reg_c, reg_f = regs[:n // 2], regs[n // 2:]
    dxc, dxf = oracle.coarse_level.dx, oracle.fine_level.dx
    padded = z_padded(oracle, fine)
    off = 0
    correction = np.zeros(oracle.shape + (4,))
    assert len(oracle.faces) == 4
    for axis, side, outside, sc, sf in oracle.faces:
        fc = sc(coarse) * dxc ** 3
        flux = sf(padded)
        a, b = flux.shape[:2]
        ff = flux.reshape(a // 2, 2, b // 2, 2, 4).sum(axis=(1, 3)) * dxf ** 3
        size = fc.size
        np.testing.assert_allclose(reg_c[off:off + size], fc.ravel(), rtol=1e-12, atol=1e-19)
        np.testing.assert_allclose(reg_f[off:off + size], ff.ravel(), rtol=1e-12, atol=1e-19)
        # the reflux is driven by the engine's own registers
        correction[outside] += side * (reg_f[off:off + size] - reg_c[off:off + size]).reshape(fc.shape) / dxc ** 3
        off += size
    assert off == n // 2
    probe(solver, 3)
    got = read(solver, 0, coarse.shape[:3])
    support = oracle.reflux_support
    T = oracle.T
    old = T.moments(coarse[support])
    old[..., 4:] = 0
    new = old.copy()
    new[..., :4] += correction[support]
    expected = coarse[support] + T.populations(new) - T.populations(old)
    np.testing.assert_allclose(got[support], expected, rtol=0, atol=POP_TOL)
    assert np.array_equal(got[~support], coarse[~support])
