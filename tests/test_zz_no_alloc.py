"""lmc_energy_noalloc: the census entry point for callers that must not
allocate device memory (e.g. code running under CUDA stream capture, where
cudaMalloc is not allowed, or hosts with a fixed memory budget). Its counters
live in a static device array shared by all calls, so two calls in a row must
each start from cleared counters and agree with lmc_energy."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_energy_matches_lmc_energy(native):
    import torch

    from latticemontecarlo_gb300 import Context, Model, synthetic as S

    el = ("Al", "Cu", "Mg", "Zn")
    coeffs = S.make_coefficients(el, 11, calibrate=False)
    ns = [10, 12]
    lattices = [S.make_lattice(ns[0], {"Al": 0.9, "Cu": 0.04, "Mg": 0.03, "Zn": 0.03}, 1, 31, el),
                S.make_lattice(ns[1], {"Al": 0.7, "Cu": 0.1, "Mg": 0.1, "Zn": 0.1}, 0, 32, el)]
    ctx = Context(Model.from_coefficients(coeffs, list(el)), device=0)
    ctx.set_lattices(ns, np.concatenate(lattices))
    expected = [ctx.energy(r)[0] for r in range(len(ns))]
    # caller-owned device buffers (allocated by the caller, never by the entry point)
    species_dev = [torch.from_numpy(sp).to("cuda:0") for sp in lattices]
    energy_dev = torch.zeros(1, dtype=torch.float64, device="cuda:0")
    torch.cuda.synchronize()
    for r in range(len(ns)):  # two calls in a row, different lattices
        native.check(native.lib.lmc_energy_noalloc(ctx._h, C.c_void_p(species_dev[r].data_ptr()), ns[r],
                                                  C.c_void_p(energy_dev.data_ptr())))
        native.check(native.lib.lmc_ctx_synchronize(ctx._h))
        got = float(energy_dev.cpu().item())
        assert got == expected[r], (r, got, expected[r])


def test_noalloc_rejects_bad_sizes(native):
    from latticemontecarlo_gb300 import Context, Model, synthetic as S

    el = ("Al", "Mg", "Zn")
    ctx = Context(Model.from_coefficients(S.make_coefficients(el, 1, calibrate=False), list(el)), device=0)
    dummy = C.c_void_p(1)
    rc = native.lib.lmc_energy_noalloc(ctx._h, dummy, 5, dummy)
    assert rc == native.LMC_ERR_UNSUPPORTED
    assert b"supercell edge" in native.lib.lmc_last_error()
