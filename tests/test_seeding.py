"""The reference's path seeding, restated: rand's StdRng::seed_from_u64 (rand 0.8.5 = ChaCha12Rng of
rand_chacha 0.3.1, keyed by rand_core 0.6.4's PCG32 seed expansion) feeding Pcg32::new_seq_offset
(crates/akari_render/src/sampler/mod.rs:157-173).

CPU: the oracle's ChaCha block function is pinned at 20 rounds by the published RFC 8439 test
vectors (the block-function test of section 2.3.2 and the keystream vectors of appendix A.1); the
oracle's sequential generator (a 4-block buffer read two words at a time, as rand_core's BlockRng
reads it) agrees with the block-indexed form the library uses on the device; the seed expansion
agrees with a plain-Python restatement of rand_core's. GPU: the library's seeds and camera rays
equal the oracle's bit for bit, for the box and the Gaussian pixel filters."""
import numpy as np
import pytest

SIGMA = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574]


def _le_words(hexbytes: str):
    b = bytes.fromhex(hexbytes.replace(" ", ""))
    return [int.from_bytes(b[4 * i:4 * i + 4], "little") for i in range(len(b) // 4)]


def test_chacha20_block_rfc8439_section_2_3_2(orc):
    key = _le_words("".join(f"{i:02x}" for i in range(32)))
    nonce = _le_words("000000090000004a00000000")
    state = SIGMA + key + [1] + nonce
    out = orc.chacha_block(state, 20)
    expect = [0xE4E7F110, 0x15593BD1, 0x1FDD0F50, 0xC47120A3, 0xC7F4D1C7, 0x0368C033, 0x9AAA2204, 0x4E6CD4C3,
              0x466482D2, 0x09AA9F07, 0x05D7C214, 0xA2028BD9, 0xD19C12B5, 0xB94E16DE, 0xE883D0CB, 0x4E3C50A2]
    assert out.tolist() == expect


@pytest.mark.parametrize("counter,stream", [
    (0, "76b8e0ada0f13d90405d6ae55386bd28bdd219b8a08ded1aa836efcc8b770dc7"
        "da41597c5157488d7724e03fb8d84a376a43b8f41518a11cc387b669b2ee6586"),
    (1, "9f07e7be5551387a98ba977c732d080dcb0f29a048e3656912c6533e32ee7aed"
        "29b721769ce64e43d57133b074d839d531ed1f28510afb45ace10a1f4b794d6f"),
])
def test_chacha20_keystream_rfc8439_appendix_a1(orc, counter, stream):
    state = SIGMA + [0] * 8 + [counter, 0, 0, 0]
    assert orc.chacha_block(state, 20).tolist() == _le_words(stream)


def _seed_from_u64_py(seed: int):
    """rand_core 0.6.4 SeedableRng::seed_from_u64 (32-byte seed) in plain Python."""
    m64 = (1 << 64) - 1
    words = []
    s = seed & m64
    for _ in range(8):
        s = (s * 6364136223846793005 + 11634580027462260723) & m64
        xs = (((s >> 18) ^ s) >> 27) & 0xFFFFFFFF
        rot = s >> 59
        words.append(((xs >> rot) | (xs << ((32 - rot) & 31))) & 0xFFFFFFFF)
    return words


@pytest.mark.parametrize("seed", [0, 1, 42, (1 << 64) - 1])
def test_seed_expansion_matches_python(orc, seed):
    assert orc.std_rng_key(seed).tolist() == _seed_from_u64_py(seed)


@pytest.mark.parametrize("seed", [0, 7])
def test_sequential_generator_matches_block_index(orc, seed):
    """gen::<u64>() number i is words (2i, 2i+1) of block i / 8 of ChaCha12 keyed by the seed."""
    key = list(orc.std_rng_key(seed))
    n = 200  # crosses several 4-block refills
    seq = orc.std_rng_u64(seed, 0, n)
    for i in range(n):
        blk = i // 8
        out = orc.chacha_block(SIGMA + key + [blk & 0xFFFFFFFF, blk >> 32, 0, 0], 12)
        w = 2 * (i % 8)
        assert int(seq[i]) == int(out[w]) | (int(out[w + 1]) << 32), i
    assert (orc.std_rng_u64(seed, 37, 50) == seq[37:87]).all()


def test_seeds_differ_between_seeds(orc):
    a, b = orc.std_rng_u64(0, 0, 64), orc.std_rng_u64(1, 0, 64)
    assert len(set(a.tolist())) == 64 and not np.intersect1d(a, b).size


@pytest.mark.gpu
@pytest.mark.parametrize("seed,first,n", [(0, 0, 5000), (1, 13, 4099), ((1 << 63) + 5, 1 << 33, 777)])
def test_device_seeds_match_oracle(sty, orc, cuda, seed, first, n):
    import torch
    out = torch.empty(n, dtype=torch.int64, device="cuda")
    sty.abi.check(sty.abi.lib().sty_std_rng_u64(seed, first, n, out.data_ptr(), None))
    torch.cuda.synchronize()
    got = out.cpu().numpy().view(np.uint64)
    assert (got == orc.std_rng_u64(seed, first, n)).all()


@pytest.mark.gpu
@pytest.mark.parametrize("filt,radius", [(0, 1.0), (0, 2.5), (1, 1.5), (1, 3.0)])
def test_camera_rays_bit_exact(sty, orc, cuda, filt, radius):
    """Depth-0 rays of every path slot (seeded streams, pixel filter, pinhole map) equal the
    oracle's restatement bit for bit, for the box and the Gaussian filters."""
    import torch
    pos, mids, mats, cam = sty.scene.cornell_box(40, 24)
    cam.filter, cam.filter_radius = filt, radius
    sc = sty.scene.Scene(pos, mids, mats, cam)
    for seed, branch in ((0, 4), (3, 2)):
        got = sc.camera_rays(branch, seed)
        torch.cuda.synchronize()
        ref = orc.camera_rays(cam, branch, seed)
        g = got.cpu().numpy()
        assert (g.view(np.uint32) == ref.view(np.uint32)).all(), np.abs(g - ref).max()
    if filt == 1:  # the Gaussian offsets stay inside [-radius, radius] and are not all clamped
        d = ref[:, 3:6]
        assert np.isfinite(d).all()
    sc.close()
