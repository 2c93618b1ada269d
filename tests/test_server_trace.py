"""Serving load generator (host only): per-job options leave the rest of a trace unchanged."""
from nbounce_gb300 import _lib as L
from nbounce_gb300 import server


def test_options_do_not_change_arrivals_sizes_or_samples():
    plain = server.make_trace(200, 30.0, 8, seed=7)
    mixed = server.make_trace(200, 30.0, 8, seed=7, options=(0, L.NB_JOB_ENV_NEE, L.NB_JOB_CACHE))
    assert [j[:4] for j in plain] == [j[:4] for j in mixed]
    assert all(j[4] == 0 for j in plain)
    flags = [j[4] for j in mixed]
    assert set(flags) == {0, L.NB_JOB_ENV_NEE, L.NB_JOB_CACHE}
    assert mixed == server.make_trace(200, 30.0, 8, seed=7, options=(0, L.NB_JOB_ENV_NEE, L.NB_JOB_CACHE))


def test_arrivals_are_increasing_and_sizes_from_the_mix():
    tr = server.make_trace(100, 10.0, 3, seed=1)
    ts = [j[0] for j in tr]
    assert ts == sorted(ts) and ts[0] > 0
    assert all(j[2] in server.RESOLUTIONS and j[3] in server.SPPS and 0 <= j[1] < 3 for j in tr)
