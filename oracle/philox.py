"""Philox4x64-10 uniform streams (oracle side; test infrastructure only).

The GPU sampler and this oracle consume the same explicit uniform stream, so
that skeleton indices can be compared bit for bit.

Stream definitions (shared with the CUDA code in ``csrc/rbrp_philox.cuh``):

* np-compat stream: the t-th uniform (t = 0, 1, ...) is
  ``(philox4x64_10(ctr=[1 + t//4, 0, 0, 0], key=[seed, 0])[t % 4] >> 11) * 2**-53``.
  This is bit-identical to ``numpy.random.Generator(numpy.random.Philox(key=seed))
  .random()``; the reference notebook draws its block samples with
  ``Generator.choice`` (``python/RBRP.ipynb`` cell 11 line 108), so with this bit
  generator the reference sampler and the GPU sampler see the same numbers.
* exponential-key stream: the uniform of original column ``c`` in block ``t``
  is ``(philox4x64_10(ctr=[1 + c//4, t + 1, ES_TAG, 0], key=[seed, 0])[c % 4] >> 11)
  * 2**-53``, i.e. ``numpy.random.Philox(key=seed, counter=[0, t+1, ES_TAG, 0])
  .random_raw(n)``.

Philox4x64-10 is the published counter-based generator of Salmon, Moraes,
Dror and Shaw (SC'11, "Parallel random numbers: as easy as 1, 2, 3"); the
multipliers and Weyl constants below are the ones published there.
"""
import numpy as np

_M64 = (1 << 64) - 1
PHILOX_M0 = 0xD2E7470EE14C6C93
PHILOX_M1 = 0xCA5A826395121157
PHILOX_W0 = 0x9E3779B97F4A7C15
PHILOX_W1 = 0xBB67AE8584CAA73B
ES_TAG = 0x4553  # 'ES': third counter word of the exponential-key stream
GEN_KEY_HI = 1   # key[1] used by the workload generators (sampler uses key[1] = 0)


def philox4x64_10(ctr, key):
    """Scalar Philox4x64 with 10 rounds; ``ctr`` is 4 words, ``key`` 2 words."""
    c = [int(x) & _M64 for x in ctr]
    k = [int(x) & _M64 for x in key]
    for r in range(10):
        if r:
            k[0] = (k[0] + PHILOX_W0) & _M64
            k[1] = (k[1] + PHILOX_W1) & _M64
        p0 = PHILOX_M0 * c[0]
        p1 = PHILOX_M1 * c[2]
        hi0, lo0 = p0 >> 64, p0 & _M64
        hi1, lo1 = p1 >> 64, p1 & _M64
        c = [hi1 ^ c[1] ^ k[0], lo1, hi0 ^ c[3] ^ k[1], lo0]
    return c


def u64_to_unit(u):
    """53-bit uniform in [0, 1), as numpy's ``next_double``."""
    return (np.asarray(u, dtype=np.uint64) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


class PhiloxStream:
    """Sequential uniform stream identical to ``Generator(Philox(key=seed)).random``.

    Keeps an explicit draw counter so tests can check that the GPU consumed
    exactly as many uniforms as the oracle.
    """

    def __init__(self, seed):
        self.seed = int(seed)
        self._gen = np.random.Generator(np.random.Philox(key=self.seed))
        self.draws = 0

    def random(self, n):
        self.draws += int(n)
        return self._gen.random(int(n))

    @property
    def generator(self):
        return self._gen


def es_uniforms(seed, block, n):
    """Uniforms of the exponential-key stream for original columns 0..n-1 of block ``block``."""
    bg = np.random.Philox(key=int(seed), counter=[0, int(block) + 1, ES_TAG, 0])
    return u64_to_unit(bg.random_raw(int(n)))
