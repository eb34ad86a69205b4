"""CPU checks of the NCE-loss oracle (oracle/nce_oracle.py): its Philox4x32-10
against the published known-answer vectors of Salmon et al. (Random123), and
its analytic FP64 gradient against FP64 central differences of its loss."""
import numpy as np
import pytest

from conftest import gmm

A, B = 0.76687364, 1.22256382


def test_philox_known_answers():
    from oracle import nce_oracle as n
    cases = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
             ((0xffffffff,) * 4, (0xffffffff, 0xffffffff),
              (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
             ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
              (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for c, k, expect in cases:
        r = n.philox4x32_10(*[np.array([v], np.uint64) for v in c], k[0], k[1])
        assert tuple(int(x[0]) for x in r) == expect


def test_noise_indices_valid():
    from oracle import nce_oracle as n
    src = np.repeat(np.arange(50), 4)
    out = n.noise_indices(src, 50, 7, seed=3, tag=1)
    assert out.shape == (200, 7) and out.min() >= 0 and out.max() < 50
    assert not np.any(out == src[:, None])


@pytest.fixture(scope="module")
def graph2k(oracle):
    X, _ = gmm(2000, 16, 8, 5.0, seed=0)
    inds, dists = oracle.knn(oracle.preprocess(X, 0), 0, 15)
    rp, cols, _ = oracle.symmetrize(inds, dists)
    return oracle.edges_from_csr(rp), cols


def test_fp64_finite_differences(graph2k):
    """The analytic gradient of the restatement equals central differences
    (FP64), on a 2000-point subset with Y ~ N(0, 1e-4 I) as in the
    differentiable-loss configuration."""
    from oracle import nce_oracle
    src, dst = graph2k
    sel = slice(0, 3000)
    src, dst = src[sel], dst[sel]
    rng = np.random.default_rng(4)
    Y = rng.normal(0, 1e-2, size=(2000, 2))
    noise = nce_oracle.noise_indices(src, 2000, 5, seed=1, tag=0)
    L, gY, gQ = nce_oracle.loss_and_grad(Y, 1.0, src, dst, noise, A, B)
    h = 1e-7
    for (r, c) in [(int(src[0]), 0), (int(dst[5]), 1), (int(noise[7, 2]), 0), (17, 1)]:
        Yp, Ym = Y.copy(), Y.copy()
        Yp[r, c] += h
        Ym[r, c] -= h
        # only the edges that touch row r depend on it
        m = (src == r) | (dst == r) | (noise == r).any(1)
        fd = (nce_oracle.loss_only(Yp, 1.0, src[m], dst[m], noise[m], A, B) -
              nce_oracle.loss_only(Ym, 1.0, src[m], dst[m], noise[m], A, B)) / (2 * h)
        assert abs(fd - gY[r, c]) <= 1e-6 * max(1.0, abs(fd)) + 1e-6
    fdq = (nce_oracle.loss_only(Y, 1.0 + 1e-6, src, dst, noise, A, B) -
           nce_oracle.loss_only(Y, 1.0 - 1e-6, src, dst, noise, A, B)) / 2e-6
    assert abs(fdq - gQ) <= 1e-6 * max(1.0, abs(fdq))


