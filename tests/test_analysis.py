"""S(k) accumulation (hermeshd_gb300/analysis.py) on fields with known spectra."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from hermeshd_gb300.analysis import StructureFactor


def test_white_noise_is_flat_at_its_variance():
    g = torch.Generator().manual_seed(0)
    sf = StructureFactor(kmax=8)
    for _ in range(40):
        sf.add_grid(0.3 * torch.randn(16, 16, 16, generator=g, dtype=torch.float64))
    r = sf.result()
    # shell k holds ~4 pi k^2 modes, half of them independent: 5 sigma bands
    for k in range(1, 8):
        n_ind = 40 * max(6, 2 * np.pi * k * k)
        assert abs(r[k] / 0.09 - 1) < 5 / np.sqrt(n_ind), (k, r[k])
    assert sf.flatness(1, 7) < 0.05


def test_single_mode_lands_in_its_shell():
    n = 32
    x = torch.arange(n, dtype=torch.float64) * 2 * np.pi / n
    f = torch.cos(3 * x)[None, None, :].expand(n, n, n) + 0 * x[:, None, None]
    sf = StructureFactor(kmax=8)
    sf.add_grid(f.contiguous())
    r = sf.result()
    assert r[3] > 1e3 * max(v for k, v in r.items() if k != 3)


def test_ensemble_boxes_of_different_sizes():
    nb, nq = 4, 11
    dims = [(8, 8, 8), (6, 6, 6)]
    sizes = [nb * nq * d[0] * d[1] * d[2] for d in dims]
    offsets = np.concatenate([[0], np.cumsum(sizes)])
    q = torch.zeros(int(offsets[-1]), dtype=torch.float64)
    g = torch.Generator().manual_seed(1)
    for i, (nx, ny, nz) in enumerate(dims):
        q[offsets[i]:offsets[i + 1]].view(nb, nq, nz, ny, nx)[0, 0] = 1 + 0.1 * torch.randn(nz, ny, nx, generator=g, dtype=torch.float64)
    sf = StructureFactor(kmax=4)
    sf.add_state(q, nb, dims, offsets)
    assert sf.samples == 2 and all(v > 0 for v in sf.result().values())
