"""The shipped surrogate weights in deployment.

sigma 10 (glsu/surrogate_sigma10.npz): on held-out sequences of the 1024^2
generator, free-running in the surrogate form, every sampled frame's phase
against the FP64 G-LS3U frame from the same reference phase: median and
90th-percentile RMSE within the 0.02 rad bar, and far below the unfiltered
least-squares phase (what the trained network gains over the method without
it).  With the network's correction reversed, the sparse probes flag the
tiles it gets wrong and the plain fallback recomputes them.

sigma 15 (glsu/surrogate_sigma15.npz): the large streaming workload's shape
(2048^2, 8 Gaussians, noise 0.05, DPRA 9x9, WFF2 sigma 15 with 31 x 31
frequencies, 512^2 tiles) on a held-out seed, within the same bar."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_shipped_network_meets_the_rmse_bar_on_held_out_seeds(glsu):
    from glsu import surrogate_eval as SE
    from glsu import train_surrogate as T
    params, dil = T.load()
    res = SE.deployment(glsu, params, dil, range(60000, 60003), nframes=40, every=20)
    print({k: v for k, v in res.items() if k != "per_frame"})
    assert res["frames_sampled"] == 6
    assert res["rmse_median"] <= 0.02 and res["rmse_p90"] <= 0.02
    assert res["rmse_without_network_median"] > 10 * res["rmse_median"]


def test_probe_flags_the_tiles_the_network_gets_wrong(glsu):
    """Probe, flag and fallback when the network is wrong: with its last
    layer negated the network misses the WFF2 phase on every tile; the
    probes flag the tiles and the plain WFF2 recomputes them, so the form's
    output is the plain frame's."""
    from glsu import surrogate_eval as SE
    from glsu import train_surrogate as T
    params, dil = T.load()
    res = SE.deployment(glsu, SE.reversed_residual(params), dil, [60100], nframes=4, every=4)
    r = res["per_frame"][0]
    print({k: v for k, v in r.items() if k != "bad_tile_rmse"})
    assert r["tiles_bad"] >= 12, "the reversed network should miss most tiles"
    assert r["tiles_bad_flagged"] >= 0.75 * r["tiles_bad"]
    assert r["tiles_flagged"] >= r["tiles_bad_flagged"]
    # recomputed tiles come from the plain WFF2: the form's error is far below the network's
    assert r["rmse"] < 0.1 * r["rmse_network_only"]


def test_sigma15_network_meets_the_rmse_bar_at_2048(glsu):
    from glsu import surrogate_eval as SE
    from glsu import train_surrogate as T
    import os
    path = os.path.join(os.path.dirname(T.__file__), "surrogate_sigma15.npz")
    params, dil = T.load(path)
    assert dil == [1, 3, 6, 12, 24, 12, 6, 1]
    res = SE.deployment(glsu, params, dil, [61000], nframes=6, every=6, size=2048, noise=0.05,
                        wff=(15.0, -1.5, 1.5, 0.1, 15.0, -1.5, 1.5, 0.1, 0.2), radius=4, tile=512, patch=4,
                        n_gauss=8)
    r = res["per_frame"][0]
    print({k: v for k, v in r.items() if k != "bad_tile_rmse"})
    assert r["rmse"] <= 0.02
    assert r["rmse_without_network"] > 10 * r["rmse"]
