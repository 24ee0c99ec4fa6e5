"""CPU checks of the numpy restatement the corrector's tensor-core kernels are
held to: its BF16 rounding against PyTorch's round-to-nearest-even
conversion and hand-made ties, and the tanh form of SiLU the kernels use."""
import numpy as np
import pytest

from test_gpu_corrector import bf16


def test_bf16_rounds_to_nearest_even():
    one = np.float32(1.0)
    cases = {
        1.0: 1.0,
        1.0 + 2.0 ** -8: 1.0,                        # tie, even neighbour below
        1.0 + 3 * 2.0 ** -8: 1.0 + 2.0 ** -6,        # tie, even neighbour above
        1.0 + 2.0 ** -8 + 2.0 ** -20: 1.0 + 2.0 ** -7,  # just past the tie
        -(1.0 + 2.0 ** -8): -1.0,
        2.0 ** -130: 2.0 ** -130,                   # subnormal, exact in bfloat16
    }
    x = np.array(list(cases), np.float32)
    np.testing.assert_array_equal(bf16(x), np.array(list(cases.values()), np.float32))
    assert bf16(np.array([one], np.float32))[0] == one


def test_bf16_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    x = np.concatenate([rng.normal(0, 1, 100000), rng.normal(0, 1e-30, 1000), rng.normal(0, 1e30, 1000)])
    x = x.astype(np.float32)
    want = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(bf16(x), want)


def test_silu_through_tanh():
    """z sigmoid(z) = h + h tanh(h), h = z / 2: the identity the kernels'
    epilogues evaluate with one hardware tanh."""
    z = np.linspace(-30, 30, 20001)
    h = 0.5 * z
    # for large negative z the tanh form cancels (|h| (1 + tanh h)): equal
    # to the rounding of |h|, far below the BF16 step the result is cut to
    np.testing.assert_allclose(h + h * np.tanh(h), z / (1 + np.exp(-z)), rtol=1e-12, atol=1e-13)
