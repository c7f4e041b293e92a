"""The oracle's multi-vacancy KMC and its Philox generator, on the CPU.

* Philox4x32-10 against the published known-answer vectors of the algorithm
  (Salmon et al., SC'11; the Random123 distribution's kat_vectors).
* With one vacancy, every traced event of orc_kmc_multi equals the reference-
  pinned single-pair predictor (orc_quartic) on the replayed lattice.
* With several vacancies (some adjacent, so environments hold a second
  vacancy): species conserved, vacancies where the trace says, and the summed
  energy changes equal the census difference under the same convention (a
  cluster with two vacancies counts nothing)."""
import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]

EL = ("Al", "Mg", "Zn")


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(oracle_mod, ctr, key, want):
    assert tuple(int(v) for v in oracle_mod.philox4x32_10(ctr, key)) == want


def _setup(oracle_mod, n, vacancies, seed, adjacent=False):
    coeffs = S.make_coefficients(EL, 7)
    sp = S.make_lattice(n, {"Al": 0.85, "Mg": 0.08, "Zn": 0.07}, vacancies, seed, EL)
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(EL, coeffs, lat)
    x = S.alphabet(EL).index("X")
    if adjacent:
        # put a second vacancy on a 1NN and a third on a 3NN site of the first
        v0 = int(np.flatnonzero(sp == x)[0])
        nb = lat.neighbors(v0)
        for j in (int(nb[0]), int(nb[20])):
            if sp[j] != x:
                other = int(np.flatnonzero((sp != x) & (np.arange(sp.size) != v0))[-1])
                sp[j], sp[other] = x, sp[j]
    return coeffs, sp, lat, m, x


def test_single_vacancy_reduces_to_the_pinned_predictor(oracle_mod):
    coeffs, sp, lat, m, x = _setup(oracle_mod, 8, 1, 3)
    start = sp.copy()
    vac = np.flatnonzero(sp == x)
    tr, vac_out, t, e = oracle_mod.kmc_multi(m, lat, sp, 450.0, 11, vac, 40)
    assert np.all(tr[:, 0] == 0)
    replay = start.copy()
    for s in range(len(tr)):
        v, tgt = int(tr[s, 1]), int(tr[s, 2])
        q = oracle_mod.quartic(m, lat, replay, v, tgt)
        assert tr[s, 4] == q[0] and tr[s, 5] == q[1]
        assert int(lat.neighbors(v)[int(tr[s, 3])]) == tgt
        replay[v], replay[tgt] = replay[tgt], x
    assert np.array_equal(replay, sp)
    assert vac_out[0] == int(tr[-1, 2]) and t == tr[-1, 7] and e == tr[-1, 8]


def test_multi_vacancy_conservation_and_energy(oracle_mod):
    coeffs, sp, lat, m, x = _setup(oracle_mod, 8, 5, 4, adjacent=True)
    m.set_vacancy_zero(True)
    start = sp.copy()
    e0, _ = oracle_mod.energy(m, lat, start)
    vac = np.flatnonzero(sp == x)
    tr, vac_out, t, e = oracle_mod.kmc_multi(m, lat, sp, 500.0, 5, vac, 60)
    assert np.array_equal(np.bincount(start, minlength=4), np.bincount(sp, minlength=4))
    assert sorted(np.flatnonzero(sp == x)) == sorted(vac_out.tolist())
    slots = vac.copy()
    for s in range(len(tr)):
        v = int(tr[s, 0])
        assert slots[v] == int(tr[s, 1])
        slots[v] = int(tr[s, 2])
    assert np.array_equal(slots, vac_out)
    assert len(set(tr[:, 0].astype(int))) > 1  # several vacancies moved
    assert np.all(np.diff(tr[:, 7]) > 0)
    e1, _ = oracle_mod.energy(m, lat, sp)
    np.testing.assert_allclose(e1 - e0, e, rtol=0, atol=1e-10)
