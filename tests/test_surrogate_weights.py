"""The shipped surrogate weights (glsu/surrogate_sigma10.npz) in deployment.

On held-out sequences of the 1024^2 generator, free-running in the surrogate
form, every sampled frame's phase against the FP64 G-LS3U frame from the
same reference phase: median and 90th-percentile RMSE within the 0.02 rad
bar, and far below the unfiltered least-squares phase (what the trained
network gains over the method without it).  With a region of noise far
outside the training range, the sparse probes flag the tiles the network
gets wrong and the plain fallback recomputes them."""
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
    from glsu import surrogate_eval as SE
    from glsu import train_surrogate as T
    params, dil = T.load()
    res = SE.deployment(glsu, params, dil, [60100], nframes=20, every=20, noise=SE.noisy_region(1024))
    r = res["per_frame"][0]
    print({k: v for k, v in r.items()})
    assert r["tiles_bad"] >= 2, "the noisy region should defeat the network on some tiles"
    assert r["tiles_bad_flagged"] >= 0.75 * r["tiles_bad"]
    # recomputed tiles come from the plain WFF2: the form's error is far below the network's
    assert r["rmse"] < 0.5 * r["rmse_network_only"]
