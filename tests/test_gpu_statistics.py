"""Flag-history distributions without the shared random stream: the GPU engine and the oracle simulate the same
gensteps with different Philox seeds, and their seqhis frequency tables must agree under a two-sample chi-squared
test (the reference's own statistical check of history tables, e.g. tests/compare_ab.py, compares runs the same way).
Bit-exact parity with a common seed is tested elsewhere; this catches a physics difference that a shared stream
could hide."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def chi2_two_sample(a, b, min_count=10):
    """Two-sample chi-squared over the history keys; rare keys are pooled.  Returns (chi2, dof, p)."""
    from scipy import stats
    keys = np.union1d(a, b)
    ca = np.array([(a == k).sum() for k in keys], dtype=np.float64)
    cb = np.array([(b == k).sum() for k in keys], dtype=np.float64)
    rare = (ca + cb) < min_count
    if rare.any():
        ca = np.r_[ca[~rare], ca[rare].sum()]
        cb = np.r_[cb[~rare], cb[rare].sum()]
    keep = (ca + cb) > 0
    ca, cb = ca[keep], cb[keep]
    na, nb = ca.sum(), cb.sum()
    ka, kb = np.sqrt(nb / na), np.sqrt(na / nb)
    chi2 = float(np.sum((ka * ca - kb * cb) ** 2 / (ca + cb)))
    dof = len(ca) - 1
    return chi2, dof, float(stats.chi2.sf(chi2, dof))


def workloads():
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    wc = G.water_cube()
    yield "water_cube", wc.arrays(), GS.water_cerenkov_gensteps(wc, 400, seed=31)
    yield "crystal_array", G.crystal_array().arrays(), GS.crystal_scint_gensteps(40, 1000, seed=32)
    ls = G.large_sphere(num_sensors=150, sphere_radius=1770.0, sensor_radius=1940.0, shell=12.0)
    yield "large_sphere_small", ls.arrays(), GS.sphere_scint_gensteps(40, 1000, seed=33, radius=1700.0)


@pytest.mark.parametrize("case", [0, 1, 2])
def test_history_table_chi2_independent_seeds(oracle, case):
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine as E
    name, arrays, gs = list(workloads())[case]
    eng = E.Engine(arrays, record_seq=1, rng_seed=0)
    eng.simulate(0, gs)
    gpu = eng.seq()["seqhis"][:, 0]
    eng.close()
    cpu_out, cpu_seq = oracle.simulate(oracle.SimConfig(arrays, seed=987654321), gs, nthreads=8)
    cpu = cpu_seq["seqhis"][:, 0]
    chi2, dof, p = chi2_two_sample(gpu, cpu)
    print("%s: %d vs %d photons, %d history classes, chi2/dof %.1f/%d, p %.3g"
          % (name, len(gpu), len(cpu), len(np.union1d(gpu, cpu)), chi2, dof, p))
    assert len(gpu) == len(cpu) and len(gpu) > 20000
    assert p > 1e-3
