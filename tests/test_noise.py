"""Range noise (rmg_noise_apply): the Philox4x32-10 generator bit-exact against the oracle (itself
pinned by the generator's published known-answer vectors), the noise arithmetic of rmagine's
GaussianNoiseCuda / RelGaussianNoiseCuda / UniformDustNoiseCuda against the binary64 oracle, and
the distributions."""
import numpy as np
import pytest

from oracle import noise as on

# Published known-answer vectors of Philox4x32-10: (counter words, key words) -> output words.
PHILOX_KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF), (0xFFFFFFFF, 0xFFFFFFFF),
     (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


# ---- CPU ---------------------------------------------------------------------------------
@pytest.mark.parametrize("case", PHILOX_KAT)
def test_oracle_philox_known_answers(case):
    c, k, want = case
    got = on.philox4x32_10(*[np.uint32(x) for x in c], np.uint32(k[0]), np.uint32(k[1]))
    assert [int(x) for x in got] == list(want)


def test_oracle_uniforms_and_normals():
    u = on.uniform01(np.array([0, 0xFF, 0x100, 0xFFFFFFFF], np.uint32))
    assert u[0] == 2.0 ** -24 and u[1] == 2.0 ** -24 and u[2] == 2.0 ** -24 and u[3] == 1 - 2.0 ** -24
    assert np.all(u.astype(np.float32).astype(np.float64) == u)  # exact in binary32
    z = on.normals(1 << 20, seed=42, call=0)
    assert abs(z.mean()) < 5e-3 and abs(z.std() - 1.0) < 5e-3
    assert abs(np.mean(z ** 4) - 3.0) < 0.05  # Gaussian kurtosis


def test_oracle_dust_probabilities():
    r = np.full(200000, 20.0, np.float32)
    out, _ = on.apply(2, r, seed=1, call=0, hit_p=0.01, ret_p=0.9)
    moved = out < 20.0
    p_hit = 1 - 0.99 ** 20
    # fraction moved = p_hit * E[0.9^(U*20)]
    e_ret = (1 - 0.9 ** 20) / (20 * -np.log(0.9))
    assert abs(moved.mean() - p_hit * e_ret) < 0.005
    assert np.all(out[moved] < 20.0) and np.all(out[moved] > 0.0)


# ---- GPU ---------------------------------------------------------------------------------
@pytest.mark.gpu
def test_philox_bits_match_the_oracle(built):
    import torch

    from rmagine_gb300 import noise

    torch.cuda.set_device(0)
    for seed, call in ((42, 0), (0x123456789ABCDEF, 7), (1, (1 << 40) + 3)):
        got = noise.philox_blocks(100003, seed, call).cpu().numpy().view(np.uint32)
        assert np.array_equal(got, on.blocks(100003, seed, call))


def _ranges(n, seed=0):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0.1, 50.0, n).astype(np.float32)
    r[::97] = 131.0  # beyond a max_range of 100
    return r


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["gaussian", "rel_gaussian"])
def test_gaussian_kinds_match_the_oracle(built, kind):
    import torch

    from rmagine_gb300 import noise

    torch.cuda.set_device(0)
    r = _ranges(1_000_003)
    opts = noise.NoiseOptions(seed=9, max_range=100.0)
    nz = noise.GaussianNoise(0.01, 0.05, opts) if kind == "gaussian" else noise.RelGaussianNoise(0.01, 0.02, 1.5, opts)
    for call in range(2):
        t = torch.from_numpy(r).cuda()
        nz.apply(t)
        got = t.cpu().numpy().astype(np.float64)
        want = on.apply(0 if kind == "gaussian" else 1, r, seed=9, call=call, mean=0.01,
                        stddev=0.05 if kind == "gaussian" else 0.02, range_exp=1.5, max_range=100.0)
        assert np.abs(got - want).max() <= 4e-6 * (1.0 + np.abs(want).max())
        assert np.array_equal(got[::97], r[::97].astype(np.float64))  # above max_range: untouched
    assert nz.call == 2


@pytest.mark.gpu
def test_dust_matches_the_oracle(built):
    import torch

    from rmagine_gb300 import noise

    torch.cuda.set_device(0)
    r = _ranges(500_001, seed=1)
    t = torch.from_numpy(r).cuda()
    noise.UniformDustNoise(0.01, 0.9, noise.NoiseOptions(seed=5, max_range=100.0)).apply(t)
    got = t.cpu().numpy().astype(np.float64)
    want, (m_hit, m_ret) = on.apply(2, r, seed=5, call=0, hit_p=0.01, ret_p=0.9, max_range=100.0)
    differ = got != want
    # a decision may flip only where the uniform sits within rounding of the probability
    assert np.all((m_hit[differ] < 1e-6) | (m_ret[differ] < 1e-6)), differ.sum()
    moved = got < r
    assert 0.05 < moved.mean() < 0.3


@pytest.mark.gpu
def test_noise_is_deterministic_tail_safe_and_unaligned(built):
    import torch

    from rmagine_gb300 import noise

    torch.cuda.set_device(0)
    r = _ranges(1003, seed=2)
    a = torch.from_numpy(r).cuda()
    noise.GaussianNoise(0.0, 0.1, noise.NoiseOptions(seed=3)).apply(a)
    base = torch.from_numpy(np.concatenate([[0.0], r]).astype(np.float32)).cuda()
    view = base[1:]  # 4-byte aligned, not 16: the scalar path, and a 3-element tail
    assert view.is_contiguous() and view.data_ptr() % 16 != 0
    noise.GaussianNoise(0.0, 0.1, noise.NoiseOptions(seed=3)).apply(view)
    assert torch.equal(a, base[1:])
    assert float(base[0]) == 0.0
    c = torch.from_numpy(r).cuda()
    n2 = noise.GaussianNoise(0.0, 0.1, noise.NoiseOptions(seed=3))
    n2.apply(c.clone())
    n2.apply(c)  # second call: different numbers
    assert not torch.equal(a, c)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["gaussian", "dust"])
def test_bulk_copy_ring_equals_register_path(built, kind):
    """A 16-byte aligned buffer streams through the bulk-copy (TMA) ring of k_noise_tma in chunks
    of 4,096 ranges (the tail through k_noise); an unaligned view of the same values goes through
    k_noise alone.  Both must give the same bits, over enough chunks that every CTA's ring wraps
    several times, and the noise status word must stay clear."""
    import torch

    from rmagine_gb300 import noise

    torch.cuda.set_device(0)
    noise.device_status(clear=True)
    n = 32 * 4096 * 1024 + 5
    g = torch.Generator(device="cuda").manual_seed(11)
    r = torch.rand(n, device="cuda", generator=g) * 120.0 + 0.5
    aligned = r.clone()
    assert aligned.data_ptr() % 16 == 0
    base = torch.empty(n + 1, device="cuda")
    base[1:] = r
    view = base[1:]
    assert view.data_ptr() % 16 != 0
    opts = noise.NoiseOptions(seed=77, max_range=100.0)
    make = (lambda: noise.GaussianNoise(0.01, 0.03, opts)) if kind == "gaussian" else \
        (lambda: noise.UniformDustNoise(0.01, 0.9, opts))
    make().apply(aligned)
    make().apply(view)
    torch.cuda.synchronize()
    assert torch.equal(aligned.view(torch.int32), view.view(torch.int32))
    assert not torch.equal(aligned, r)
    assert noise.device_status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("n", [4096, 3 * 4096, 4096 * 997, 4096 * 997 + 4, 4096 * 997 + 4095])
def test_chunk_boundaries_match_the_oracle(built, n):
    """Sizes at and around whole chunks of the bulk-copy ring, against the oracle."""
    import torch

    from rmagine_gb300 import noise

    torch.cuda.set_device(0)
    r = _ranges(n, seed=n % 1000)
    t = torch.from_numpy(r).cuda()
    noise.GaussianNoise(0.0, 0.05, noise.NoiseOptions(seed=4, max_range=100.0)).apply(t)
    got = t.cpu().numpy().astype(np.float64)
    want = on.apply(0, r, seed=4, call=0, mean=0.0, stddev=0.05, max_range=100.0)
    assert np.abs(got - want).max() <= 4e-6 * (1.0 + np.abs(want).max())
    assert noise.device_status() == 0
