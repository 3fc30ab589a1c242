"""Seed geometry kernels (csrc/seeds.cu).

CPU: the closed-form rank that qsl_tile_order scatters each seed to is the
seed's position in the sort of the tile keys (the order the framework-side
argsort used to produce), on random stack shapes with ragged edge tiles and
plane groups.  GPU: qsl_tile_order equals that argsort on the device, and
qsl_plane_seeds equals the seed-grid expression evaluated one array
operation at a time in double, bit for bit."""
import numpy as np
import pytest


def tile_keys(nplanes, n0, n1, ty, tx, g, xp=np):
    p = xp.arange(nplanes).reshape(-1, 1, 1)
    y = xp.arange(n0).reshape(1, -1, 1)
    x = xp.arange(n1).reshape(1, 1, -1)
    ntx, nty = (n1 + tx - 1) // tx, (n0 + ty - 1) // ty
    return (((((p // g) * nty + y // ty) * ntx + x // tx) * g + p % g) * (ty * tx) + (y % ty) * tx +
            (x % tx)).reshape(-1)


def closed_form_order(nplanes, n0, n1, ty, tx, g):
    """The rank formula of k_tile_order, restated."""
    q = np.arange(nplanes * n0 * n1)
    x, r = q % n1, q // n1
    y, p = r % n0, r // n0
    pg, pp, ti, tj = p // g, p % g, y // ty, x // tx
    G = np.minimum(g, nplanes - pg * g)
    h = np.minimum(ty, n0 - ti * ty)
    w = np.minimum(tx, n1 - tj * tx)
    rank = pg * g * n0 * n1 + G * ti * ty * n1 + G * h * tj * tx + pp * h * w + (y % ty) * w + x % tx
    out = np.full(q.size, -1)
    out[rank] = q
    return out


def shapes(seed, count):
    rng = np.random.default_rng(seed)
    for _ in range(count):
        npl, n0, n1 = int(rng.integers(1, 6)), int(rng.integers(1, 40)), int(rng.integers(1, 40))
        yield npl, n0, n1, int(rng.integers(1, 10)), int(rng.integers(1, 10)), int(rng.integers(1, npl + 1))


def test_closed_form_rank_is_the_sorted_order():
    for npl, n0, n1, ty, tx, g in shapes(0, 400):
        ref = np.argsort(tile_keys(npl, n0, n1, ty, tx, g), kind="stable")
        assert (closed_form_order(npl, n0, n1, ty, tx, g) == ref).all(), (npl, n0, n1, ty, tx, g)


@pytest.mark.gpu
def test_tile_order_kernel_equals_sorted_keys(cuda):
    import torch
    from fastqsl_gb300 import api
    for npl, n0, n1, ty, tx, g in list(shapes(1, 60)) + [(128, 258, 258, 8, 8, 128), (3, 1024, 1024, 16, 16, 1)]:
        got = api.tile_order(npl, n0, n1, ty, tx, cuda, plane_group=g)
        ref = torch.argsort(tile_keys(npl, n0, n1, ty, tx, g, xp=_TorchArange(cuda))).to(torch.int32)
        assert torch.equal(got, ref), (npl, n0, n1, ty, tx, g)


class _TorchArange:
    """numpy's arange/reshape spelled for tile_keys on torch device tensors."""

    def __init__(self, device):
        self.device = device

    def arange(self, n):
        import torch
        return torch.arange(n, device=self.device, dtype=torch.int64)


@pytest.mark.gpu
def test_plane_seeds_kernel_equals_array_expression(cuda):
    import torch
    from fastqsl_gb300 import api, serving
    rng = np.random.default_rng(5)
    for _ in range(12):
        n0, n1, npl = int(rng.integers(3, 90)), int(rng.integers(3, 90)), int(rng.integers(1, 5))
        normal = rng.normal(size=3)
        n, u, v = serving.plane_axes(normal)
        c = rng.uniform(-50, 400, 3)
        s = float(rng.uniform(0.05, 2.0))
        # the expression, one array operation at a time in double
        C = torch.tensor(c, dtype=torch.float64, device=cuda)
        j = (torch.arange(n1, dtype=torch.float64, device=cuda) - (n1 - 1) / 2.0) * s
        i = (torch.arange(n0, dtype=torch.float64, device=cuda) - (n0 - 1) / 2.0) * s
        k = torch.arange(npl, dtype=torch.float64, device=cuda) * s
        U, V, N = (torch.tensor(a, dtype=torch.float64, device=cuda) for a in (u, v, n))
        pts = (C.view(1, 1, 1, 3) + k.view(-1, 1, 1, 1) * N + i.view(1, -1, 1, 1) * V + j.view(1, 1, -1, 1) * U)
        pts = pts.reshape(-1, 3).to(torch.float32)
        xs, ys, zs = api.plane_seeds(c, n, u, v, s, n0, n1, npl, device=cuda)
        torch.cuda.synchronize()
        for a, col in zip((xs, ys, zs), range(3)):
            assert torch.equal(a, pts[:, col].contiguous())
