"""Known-answer test of the Philox4x32-10 generator (Salmon et al., SC'11).

Every stochastic stage of the kernels (order draws, scatter angles, the
CAT stack's draws, photon generation, pose wiggles) draws from the device
function ``philox4x32_10``.  Distribution tests cannot tell a wrong round
constant or key schedule from a right one, so the device function is held
to the published Random123 Philox4x32-10 known-answer vectors (the zero
counter and key, the all-ones counter and key, and the pi-digit counter
and key), and to a Python restatement of the published algorithm on
random inputs.  The CPU part checks the restatement itself against the
vectors and that a one-bit change to a round constant breaks them.
"""
import numpy as np
import pytest

M0, M1 = 0xD2511F53, 0xCD9E8D57           # round multipliers
W0, W1 = 0x9E3779B9, 0xBB67AE85           # Weyl key increments

# (counter words, key words) -> output words, Random123's kat_vectors for philox4x32_10
KAT = [((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
        (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
       ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
        (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
       ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
        (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]


def philox(ctr, key, m0=M0, m1=M1, w0=W0, w1=W1, rounds=10):
    """Philox4x32: per round two 32x32->64 products, the S-box
    (hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0) and the Weyl key bump."""
    c = [int(v) for v in ctr]
    k = [int(v) for v in key]
    for _ in range(rounds):
        p0, p1 = m0 * c[0], m1 * c[2]
        c = [(p1 >> 32) ^ c[1] ^ k[0], p1 & 0xffffffff, (p0 >> 32) ^ c[3] ^ k[1], p0 & 0xffffffff]
        k = [(k[0] + w0) & 0xffffffff, (k[1] + w1) & 0xffffffff]
    return tuple(c)


def test_restatement_reproduces_published_vectors():
    for ctr, key, want in KAT:
        assert philox(ctr, key) == want


@pytest.mark.parametrize('which', ['m0', 'm1', 'w0', 'w1'])
def test_one_bit_in_a_constant_breaks_the_vectors(which):
    kw = {'m0': M0, 'm1': M1, 'w0': W0, 'w1': W1}
    kw[which] ^= 1 << 7
    assert all(philox(ctr, key, **kw) != want for ctr, key, want in KAT)


def _device(inp):
    import torch
    from marxs_gb300 import _abi
    lib = _abi.load()
    x = torch.from_numpy(np.ascontiguousarray(inp, dtype=np.uint32).view(np.int32)).cuda()
    out = torch.zeros((len(inp), 4), dtype=torch.int32, device='cuda')
    rc = lib.mgpu_philox4x32_10(x.data_ptr(), out.data_ptr(), len(inp),
                                torch.cuda.current_stream().cuda_stream)
    assert rc == 0
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint32)


@pytest.mark.gpu
def test_device_generator_known_answers():
    inp = np.array([list(c) + list(k) for c, k, _ in KAT], dtype=np.uint32)
    got = _device(inp)
    for row, (_, _, want) in zip(got, KAT):
        assert tuple(int(v) for v in row) == want


@pytest.mark.gpu
def test_device_generator_equals_restatement():
    rng = np.random.default_rng(2026)
    inp = rng.integers(0, 2 ** 32, size=(4096, 6), dtype=np.uint64).astype(np.uint32)
    got = _device(inp)
    for k in range(0, 4096, 37):
        assert tuple(int(v) for v in got[k]) == philox(inp[k, :4], inp[k, 4:])
