"""Statistics of the stochastic stress (random.f90:106-145 with the MKL
stream replaced by Philox-4x32-10; the six independent entries of the
symmetrised normal matrix drawn directly).  The reference pins no random value (its
call is disabled, flux.f90:41): these are the distributional checks, on the
oracle's generator, which the CUDA kernels match (tests/test_parity_gpu.py,
noisy cases)."""
import numpy as np
import pytest

import oracle as O

N = 20000


def _samples(eta=1.0, zeta=0.0, kind=3, step=7, stage=1):
    G = np.zeros((N, 6))
    S = np.zeros((N, 6))
    for i in range(N):
        G[i], S[i] = O.noise_sample(1234, step, stage, kind, i // 8, i % 8, eta, zeta)
    return G, S


@pytest.fixture(scope="module")
def samples():
    return _samples()


def test_normals_moments(samples):
    G, _ = samples
    z = G.flatten()
    se = 1.0 / np.sqrt(z.size)
    assert abs(z.mean()) < 5 * se
    assert abs(z.var() - 1.0) < 5 * np.sqrt(2.0) * se
    assert abs((z ** 4).mean() - 3.0) < 0.1               # Gaussian kurtosis
    C = np.corrcoef(G.T)
    assert np.abs(C - np.eye(6)).max() < 5 / np.sqrt(N)   # independent components


def test_normals_gaussian_ks(samples):
    stats = pytest.importorskip("scipy.stats")
    G, _ = samples
    assert stats.kstest(G.flatten(), "norm").pvalue > 1e-3


def test_stress_covariance(samples):
    _, S = samples
    # S = eta (sym G - tr G/3): var Sxx = 2/3, cov(Sxx, Syy) = -1/3, var Sxy = 1, traceless
    assert np.abs(S[:, 0] + S[:, 1] + S[:, 2]).max() < 1e-12
    C = np.cov(S.T)
    tol = 6 / np.sqrt(N)
    assert abs(C[0, 0] - 2 / 3) < tol and abs(C[1, 1] - 2 / 3) < tol and abs(C[2, 2] - 2 / 3) < tol
    assert abs(C[0, 1] + 1 / 3) < tol and abs(C[0, 2] + 1 / 3) < tol
    assert abs(C[3, 3] - 1) < tol and abs(C[4, 4] - 1) < tol and abs(C[5, 5] - 1) < tol
    assert abs(C[3, 4]) < tol and abs(C[0, 3]) < tol


def test_bulk_part_and_amplitudes():
    G, S = _samples(eta=0.5, zeta=0.2)
    tr = S[:, 0] + S[:, 1] + S[:, 2]
    assert np.allclose(tr, 3 * 0.2 * (G[:, 0] + G[:, 1] + G[:, 2]), atol=1e-12)
    assert abs(np.var(S[:, 3]) - 0.25) < 6 * 0.25 / np.sqrt(N)


def test_counters_give_distinct_streams():
    a = [O.noise_sample(1, 0, 0, 0, 5, 0)[0] for _ in range(2)]
    assert np.array_equal(a[0], a[1])                         # deterministic
    variants = [O.noise_sample(*args)[0] for args in
                ((1, 0, 0, 0, 5, 0), (2, 0, 0, 0, 5, 0), (1, 1, 0, 0, 5, 0), (1, 0, 1, 0, 5, 0),
                 (1, 0, 0, 1, 5, 0), (1, 0, 0, 0, 6, 0), (1, 0, 0, 0, 5, 1))]
    for i in range(len(variants)):
        for j in range(i + 1, len(variants)):
            assert not np.allclose(variants[i], variants[j])


def test_philox_known_answers():
    """Philox-4x32-10 known-answer vectors of the generator's authors
    (Random123 kat_vectors: zero, all-ones and pi-digit counters/keys)."""
    import oracle as O
    kat = [
        ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
        ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
        ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
         (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
    ]
    for ctr, key, want in kat:
        assert O.philox4x32_10(ctr, key) == list(want)
