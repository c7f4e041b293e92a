"""lmc_energy_noalloc: the census entry point for callers that cannot allocate
device memory at the call site (a host whose own pool allocator owns the GPU's
memory, a fixed memory budget, a loop where cudaMalloc would synchronise the
device). Its counters live in a static device array shared by all calls, so two
calls in a row must each start from cleared counters and agree with
lmc_energy; a species code outside the alphabet must give NaN, not a fault,
and leave the next call unaffected."""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case():
    from latticemontecarlo_gb300 import Context, Model, synthetic as S

    el = ("Al", "Cu", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 11, calibrate=False)
    ns = [10, 12]
    lattices = [S.make_lattice(ns[0], {"Al": 0.9, "Cu": 0.04, "Mg": 0.03, "Zn": 0.03}, 1, 31, el),
                S.make_lattice(ns[1], {"Al": 0.7, "Cu": 0.1, "Mg": 0.1, "Zn": 0.1}, 0, 32, el)]
    ctx = Context(Model.from_coefficients(coeffs, list(el)), device=0)
    ctx.set_lattices(ns, np.concatenate(lattices))
    return ctx, ns, lattices


def _noalloc(native, ctx, species_dev, n, energy_dev):
    native.check(native.lib.lmc_energy_noalloc(ctx._h, C.c_void_p(species_dev.data_ptr()), n,
                                              C.c_void_p(energy_dev.data_ptr())))
    native.check(native.lib.lmc_ctx_synchronize(ctx._h))
    return float(energy_dev.cpu().item())


def test_noalloc_energy_matches_lmc_energy(native):
    import torch

    ctx, ns, lattices = _case()
    expected = [ctx.energy(r)[0] for r in range(len(ns))]
    # caller-owned device buffers (allocated by the caller, never by the entry point)
    species_dev = [torch.from_numpy(sp).to("cuda:0") for sp in lattices]
    energy_dev = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    for r in range(len(ns)):  # two calls in a row, different lattices
        got = _noalloc(native, ctx, species_dev[r], ns[r], energy_dev)
        assert got == expected[r], (r, got, expected[r])


def test_noalloc_bad_species_code_gives_nan(native):
    import torch

    ctx, ns, lattices = _case()
    expected = ctx.energy(0)[0]
    energy_dev = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    for bad in (5, -1, 127):  # the alphabet has 5 codes (Al Cu Mg X Zn)
        sp = lattices[0].copy()
        sp[1234] = bad
        got = _noalloc(native, ctx, torch.from_numpy(sp).to("cuda:0"), ns[0], energy_dev)
        assert math.isnan(got), (bad, got)
        # the shared counters and the bad-code word are cleared by the next call
        good = _noalloc(native, ctx, torch.from_numpy(lattices[0]).to("cuda:0"), ns[0], energy_dev)
        assert good == expected


def test_noalloc_rejects_bad_sizes(native):
    from latticemontecarlo_gb300 import Context, Model, synthetic as S

    el = ("Al", "Mg", "Zn")
    ctx = Context(Model.from_coefficients(S.make_coefficients(el, 1, calibrate=False), list(el)), device=0)
    dummy = C.c_void_p(1)
    rc = native.lib.lmc_energy_noalloc(ctx._h, dummy, 5, dummy)
    assert rc == native.LMC_ERR_UNSUPPORTED
    assert b"supercell edge" in native.lib.lmc_last_error()
