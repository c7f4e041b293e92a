"""CanonicalMcOmp's batch order on the reference's mt19937_64 stream (LMC_CMC_REFERENCE_BATCH)
against the oracle's restatement, for batch sizes on either side of the kernel's 32-pair steps
(the batch build takes the stream's different-species pairs a set at a time, the Metropolis tests
run 32 pairs at once): final lattice, attempts, acceptances and the energy before every attempt.
ECIs scaled so |dE| ~ kT: the test rejects often."""
import ctypes as C

import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

EL = ("Al", "Cu", "Mg", "Zn")
FRAC = {"Al": 0.88, "Cu": 0.04, "Mg": 0.04, "Zn": 0.04}


def _run(native, ctx, T, attempts, seed, batch, energy):
    cap = attempts + 4 * batch
    trace = np.zeros(cap)
    opt = native.CmcOptions(native.LMC_CMC_REFERENCE_BATCH, seed, batch, 0,
                            trace.ctypes.data_as(C.POINTER(C.c_double)))
    e = C.c_double(energy)
    done, acc = C.c_uint64(), C.c_uint64()
    native.check(native.lib.lmc_cmc_run(ctx._h, 0, T, attempts, C.byref(opt), C.byref(e), C.byref(done),
                                        C.byref(acc)))
    return e.value, done.value, acc.value, trace[:done.value]


@pytest.mark.parametrize("batch", [1, 5, 33, 64])
def test_reference_batch_against_oracle(native, oracle_mod, golden, batch):
    from latticemontecarlo_gb300 import api
    G, _ = golden
    coeffs = G.scaled_eci(S.make_coefficients(EL, 17), 800.0)
    n, T, seed = 12, 500.0, 29 + batch
    sp = S.make_lattice(n, FRAC, 0, 5, EL)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(EL, coeffs, lat)
    ref = sp.copy()
    attempts = 40 * batch + 1500
    r_done, r_e, r_acc, r_tr = oracle_mod.cmc(m, lat, ref, T, seed, attempts, batch, 0.0, trace=True)
    ctx = api.Context(api.Model.from_coefficients(coeffs, list(EL)))
    ctx.set_lattices([n], sp)
    e, done, acc, tr = _run(native, ctx, T, attempts, seed, batch, 0.0)
    assert done == r_done and acc == r_acc
    assert np.array_equal(ctx.get_lattices(), ref)
    np.testing.assert_allclose(tr, r_tr, rtol=0, atol=1e-12)
    np.testing.assert_allclose(e, r_e, rtol=0, atol=1e-12)
    assert 0.2 < acc / done < 0.9, acc / done
