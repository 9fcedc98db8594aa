"""Channel extraction on seeded random track layouts
(Channel_extractor_5, sfxc/src/channel_extractor_5.cc:27-99): 32- and 64-bit
words, 1- and 2-bit samples, fan-out 1, 2, 4 or 8 (at most 8 tracks a
subband), 1 to 16 subbands (the counts that extractor takes) whose tracks are a random choice of the word's
bits in random order.

CPU: the restatement against the reference's own extractor.
GPU: the library's extraction kernel against the restatement.
Both bit-exact."""
import numpy as np
import pytest

N_LAYOUTS = 24


def random_layout(seed):
    rng = np.random.Generator(np.random.PCG64(7000 + seed))
    word_bytes = int(rng.choice([4, 4, 8]))
    bits = int(rng.choice([1, 2]))
    # at most 8 tracks a subband: one output byte per word and subband at most
    # (Channel_extractor_5 packs 8 / tracks samples per output byte)
    fan_out = int(rng.choice([f for f in (1, 2, 4, 8) if f * bits <= 8]))
    per = bits * fan_out
    # the reference's Channel_extractor_5 takes 1, 2, 4, 8 or 16 subbands
    n_sub = int(rng.choice([n for n in (1, 2, 4, 8, 16) if n * per <= word_bytes * 8]))
    chosen = rng.permutation(word_bytes * 8)[:n_sub * per]
    tracks = [[int(x) for x in chosen[i * per:(i + 1) * per]] for i in range(n_sub)]
    nwords = 8 * int(rng.integers(16, 200))
    words = rng.integers(0, 256, size=nwords * word_bytes, dtype=np.uint8).tobytes()
    return words, word_bytes, bits, nwords, tracks


@pytest.fixture(scope="module")
def reference_available():
    from oracle import build_ref
    if build_ref.build() is None:
        pytest.skip("reference checkout not available")


@pytest.mark.parametrize("seed", range(N_LAYOUTS))
def test_restatement_matches_reference(seed, reference_available):
    from oracle import jobs
    words, wb, bits, nwords, tracks = random_layout(seed)
    assert jobs.extract(words, wb, bits, nwords, tracks, impl="oracle") == jobs.extract(words, wb, bits, nwords,
                                                                                         tracks)


@pytest.mark.gpu
def test_gpu_matches_restatement(gpu_node, oracle_exe):
    from oracle import jobs
    for seed in range(N_LAYOUTS):
        words, wb, bits, nwords, tracks = random_layout(seed)
        want = jobs.extract(words, wb, bits, nwords, tracks, impl="oracle")
        assert [bytes(x) for x in gpu_node.extract_channels(words, wb, bits, tracks)] == want, seed
