"""curl B on the GPU (qsl_curl_grid through fastqslpy.FastQSL.curl_of_B_grid)
bit for bit against the reference's own curl_of_B_grid (golden fixture)."""
import numpy as np
import pytest
import torch

import golden_util as G

pytestmark = pytest.mark.gpu


def test_curl_matches_reference(cuda):
    from fastqsl_gb300 import synthetic as S
    from fastqsl_gb300.fastqslpy import FastQSL
    g, meta = G.load("curl_stretch.npz")
    spec = S.bipole4_stretch(meta["seed"], shape=tuple(meta["shape"]))
    xa, ya, za = S.stretched_axes(spec.shape, z_ratio=meta["z_ratio"])
    Bx, By, Bz = S.make_field_coords(spec, xa, ya, za)
    cur = FastQSL.curl_of_B_grid(*[torch.from_numpy(b) for b in (Bx, By, Bz)], xa, ya, za)
    torch.cuda.synchronize()
    for c, k in zip(cur, ("curl_x", "curl_y", "curl_z")):
        assert c.stride() == (1, Bx.shape[0], Bx.shape[0] * Bx.shape[1])
        np.testing.assert_array_equal(c.cpu().numpy(), g[k])
