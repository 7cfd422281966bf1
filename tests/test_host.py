"""Host-side helpers of the package against the oracle (no GPU)."""
import importlib

import numpy as np

from fixtures import M, l_prism, square_torus, stairs

conc = importlib.import_module("cuacd-web_gb300.concave")
gen = importlib.import_module("cuacd-web_gb300.meshgen")
part = importlib.import_module("cuacd-web_gb300.part")


def test_concave_planes_match_oracle(oracle):
    for m, n in ((l_prism(), 8), (stairs(), 16), (gen.staircase(8), 16), (square_torus(), 4), (M.unit_cube(), 8)):
        a = conc.concave_edge_planes(m, n)
        b = oracle.concave_planes(m, n)
        assert a.shape == b.shape
        assert np.allclose(a, b, atol=1e-6)


def test_concave_reservoir_matches_oracle(oracle):
    """More concave edges than reservoir slots exercises the seeded LCG."""
    m = gen.staircase(12)
    for seed in (12345, 7, 99):
        a = conc.concave_edge_planes(m, 4, seed=seed)
        b = oracle.concave_planes(m, 4, seed=seed)
        assert np.allclose(a, b, atol=1e-6)


def test_rv_cost_matches_oracle(oracle):
    # the engine's volumes are float32: compare on float32-rounded inputs
    for mv, hv in ((1.0, 1.0), (0.5, 0.75), (0.1, 0.1000001), (2.0, 1.0), (1e-6, 1.0)):
        mv, hv = float(np.float32(mv)), float(np.float32(hv))
        assert abs(part.rv_cost(mv, hv) - oracle.rv_cost(mv, hv)) < 1e-6


def test_generators_closed():
    for m in (gen.staircase(4), gen.staircase(8), gen.staircase(16), gen.noisy_icosphere(3)):
        assert M.is_closed(m) and M.signed_volume(m) > 0
    assert gen.icosphere(4).nv == 2562 and gen.icosphere(4).nt == 5120
