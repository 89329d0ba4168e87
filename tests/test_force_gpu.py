"""All-pairs force on the GPU against the oracle and the reference's golden
vectors.  Tolerances: the exact form is bit-identical; the fast FP64 form
agrees to 1e-13 relative per body (the stated bar); the naive form to 1e-12."""
import numpy as np
import pytest

from abie_gb300 import ics
from conftest import rel_err_per_body

G = ics.G_SOLAR
pytestmark = pytest.mark.gpu
CASES = ["force_sys", "force_edge", "force_disk", "force_n1", "force_n2", "force_n3"]


@pytest.mark.parametrize("case", CASES)
def test_exact_is_bit_identical_to_reference(clib, golden, case):
    p, m = golden[case + "_pos"], golden[case + "_m"]
    assert np.array_equal(clib.force(p, m, G, "exact"), golden[case + "_acc"])


@pytest.mark.parametrize("case", CASES)
def test_fp64_within_1e13(clib, golden, case):
    p, m = golden[case + "_pos"], golden[case + "_m"]
    assert rel_err_per_body(clib.force(p, m, G, "fp64"), golden[case + "_acc"]) <= 1e-13


def test_naive_matches_offload_semantics(clib, golden):
    p, m = golden["force_sys_pos"], golden["force_sys_m"]
    assert rel_err_per_body(clib.force(p, m, G, "naive"), golden["force_sys_acc"]) <= 1e-12


def test_reference_entry_point_uses_current_form(clib, golden):
    p, m = golden["force_disk_pos"], golden["force_disk_m"]
    old = clib.set_force_mode("exact")
    try:
        acc = clib.ode_n_body_second_order(p, m.size, G, m)
    finally:
        clib.set_force_mode(old)
    assert np.array_equal(acc, golden["force_disk_acc"])


def test_full_size_disk_fp64(clib, oracle):
    """16,385-body workload: fast FP64 vs the oracle on a sample of sinks."""
    p, v, m, r = ics.planetesimal_disk()
    acc = clib.force(p, m, G, "fp64")
    sinks = np.r_[0:64, 8000:8064, m.size - 64:m.size]
    ref = np.zeros(p.size)
    for lo in (0, 8000, m.size - 64):
        oracle.force(p, m, G, j0=lo, j1=lo + 64, acc=ref, threads=8)
    idx = (3 * sinks[:, None] + np.arange(3)).reshape(-1)
    assert rel_err_per_body(acc[idx], ref[idx]) <= 1e-13


def test_exact_vs_oracle_cfg1(clib, oracle):
    p, v, m, r = ics.planetary_system()
    assert np.array_equal(clib.force(p, m, G, "exact"), oracle.force(p, m, G))


def test_fp64_shapes_agree(clib):
    """Every lanes-per-sink / source-chunk shape gives the same sums to 1e-13."""
    p, v, m, r = ics.planetesimal_disk(seed=5, n=3000)
    base = clib.force(p, m, G, "exact")
    lib = clib.lib
    try:
        for lanes in (1, 8, 32):
            for chunks in (1, 3):
                lib.abie_debug_force_shape(lanes, chunks)
                assert rel_err_per_body(clib.force(p, m, G, "fp64"), base) <= 1e-13
    finally:
        lib.abie_debug_force_shape(0, 0)


def test_energy_matches_reference(clib, golden):
    e = clib.energy(golden["force_disk_pos"], golden["energy_disk_vel"], golden["force_disk_m"], G)
    assert abs(e - golden["energy_disk"][0]) <= 1e-14 * abs(golden["energy_disk"][0])


def test_zero_and_one_body(clib):
    assert clib.force(np.zeros(3), np.ones(1), G, "fp64").tolist() == [0.0, 0.0, 0.0]
    assert clib.force(np.zeros(0), np.zeros(0), G, "fp64").size == 0


def test_large_mixed_masses_parallel_compaction(clib, oracle):
    """10,000 bodies (the many-block source compaction) with massless,
    deleted (negative) and massive bodies interleaved at random: the exact
    form equals the oracle bit for bit (the source list keeps body order),
    the fast form agrees to 1e-13, and deleted sinks read zero."""
    p, v, m, r = ics.planetary_system(seed=17, n_planets=8, n_tp=9991)
    rng = np.random.default_rng(17)
    kind = rng.integers(0, 3, m.size)
    m = m.copy()
    m[1:] = np.where(kind[1:] == 0, 10 ** rng.uniform(-9, -5, m.size - 1),
                     np.where(kind[1:] == 1, 0.0, -1.0))
    ref = oracle.force(p, m, G, threads=8)
    assert np.array_equal(clib.force(p, m, G, "exact"), ref)
    fast = clib.force(p, m, G, "fp64")
    live = np.repeat(m >= 0, 3)
    assert np.all(fast[~live] == 0.0)
    assert rel_err_per_body(fast[live], ref[live]) <= 1e-13


@pytest.mark.parametrize("n", [8192, 8200, 131072, 131073])
def test_symmetric_form_sizes(clib, oracle, n):
    """All-massive systems about the symmetric form's limits: 8,192 bodies
    (its first size), 8,200 (a partial last tile of 32), 131,072 (its last
    size) and 131,073 (the chunked form again).  The fast form agrees with
    the exact one on every sink to 1e-13 at the smaller sizes and with the
    oracle on sampled sinks at the larger ones, and a second call gives the
    same doubles (the partial sums are added in a fixed order)."""
    p, v, m, r = ics.planetesimal_disk(seed=40 + n % 97, n=n - 1)
    fast = clib.force(p, m, G, "fp64")
    assert np.array_equal(clib.force(p, m, G, "fp64"), fast)
    if n <= 8200:
        assert rel_err_per_body(fast, clib.force(p, m, G, "exact")) <= 1e-13
        return
    ref = np.zeros(p.size)
    los = (0, n // 2 - 17, n - 64)
    for lo in los:
        oracle.force(p, m, G, j0=lo, j1=lo + 64, acc=ref, threads=8)
    sinks = np.concatenate([np.arange(lo, lo + 64) for lo in los])
    idx = (3 * sinks[:, None] + np.arange(3)).reshape(-1)
    assert rel_err_per_body(fast[idx], ref[idx]) <= 1e-13


def _energy_terms_fsum(p, v, m, G):
    """The reference's energy terms (src/common.c:340-357), each rounded as
    the reference rounds it, summed exactly (math.fsum)."""
    import math
    p, v = p.reshape(-1, 3), v.reshape(-1, 3)
    terms = []
    for i in range(m.size):
        if m[i] == 0.0:
            continue
        s = v[i, 0] * v[i, 0]
        s = s + v[i, 1] * v[i, 1]
        s = s + v[i, 2] * v[i, 2]
        nv = np.sqrt(s)
        terms.append(0.5 * m[i] * (nv * nv))
        j = np.array([k for k in range(m.size) if k != i and m[k] != 0.0], dtype=int)
        if j.size:
            d = p[i] - p[j]
            r2 = d[:, 0] * d[:, 0]
            r2 = r2 + d[:, 1] * d[:, 1]
            r2 = r2 + d[:, 2] * d[:, 2]
            c = 0.5 * G * m[i]
            terms.extend((-((c * m[j]) / np.sqrt(r2))).tolist())
    return math.fsum(terms), math.fsum(abs(t) for t in terms)


@pytest.mark.parametrize("n", [1, 2, 7, 9, 33, 300])
def test_energy_sums_the_reference_terms(clib, n):
    """One warp per body, double-double sums: the energy equals the exact
    sum of the reference's own rounded terms to about one rounding of the
    result, with massless and negative-mass bodies mixed in and sizes that
    leave blocks of 8 warps part-filled."""
    rng = np.random.default_rng(700 + n)
    p = rng.normal(0.0, 5.0, 3 * n)
    v = rng.normal(0.0, 2.0, 3 * n)
    m = 10 ** rng.uniform(-9, -3, n)
    if n > 2:
        m[rng.integers(0, n, max(1, n // 5))] = 0.0
        m[rng.integers(0, n, max(1, n // 7))] *= -1.0
    e = clib.energy(p, v, m, G)
    exact, scale = _energy_terms_fsum(p, v, m, G)
    assert abs(e - exact) <= 2.0 * np.spacing(abs(exact)) + 1e-28 * scale
