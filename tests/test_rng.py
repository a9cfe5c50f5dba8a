"""The sample streams, bit for bit: the reference's PCG hash, hash-based
Owen scrambling of Sobol's first two dimensions, per-dimension keys and the
golden-ratio spectrum position (src/shaders.mjs:135-212, 1857-1859), seeded
as main() seeds a camera path (:1852-1856), light_trace() a photon (:1638)
and photon_gather() a pixel (:1585).

A numpy restatement written here straight from the shader pins the oracle's
streams (CPU); the CUDA kernels' streams, drawn through the product's own
seeding functions (raymond_sample_streams), must equal the oracle's bit for
bit (GPU). Integer work: no tolerance."""

import ctypes

import numpy as np
import pytest

import oracle

M = np.uint64(0xFFFFFFFF)


def u32(x):
    return (np.asarray(x, dtype=np.uint64) & M).astype(np.uint64)


def pcg(v):
    state = u32(u32(v) * np.uint64(747796405) + np.uint64(2891336453))
    word = u32((((state >> ((state >> np.uint64(28)) + np.uint64(4))) ^ state)) * np.uint64(277803737))
    return u32((word >> np.uint64(22)) ^ word)


def reverse_bits(x):
    x = u32(x)
    out = np.zeros_like(x)
    for b in range(32):
        out |= ((x >> np.uint64(b)) & np.uint64(1)) << np.uint64(31 - b)
    return out


def owen(x, seed):
    seed = u32(seed)
    v = reverse_bits(x)
    v = u32(v ^ u32(v * np.uint64(0x3D20ADEA)))
    v = u32(v + seed)
    v = u32(v * ((seed >> np.uint64(16)) | np.uint64(1)))
    v = u32(v ^ u32(v * np.uint64(0x05526C56)))
    v = u32(v ^ u32(v * np.uint64(0x53A22864)))
    return reverse_bits(v)


def sobol2(i):
    i = u32(i)
    r = np.zeros_like(i)
    v = np.full_like(i, 0x80000000)
    for _ in range(32):
        r = np.where(i & np.uint64(1), r ^ v, r)
        i = i >> np.uint64(1)
        v = v ^ (v >> np.uint64(1))
    return r


def unit(x):
    return (u32(x) >> np.uint64(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)


def reference_streams(pairs, dim_ids, chain, seed_hash=0):
    """The shader's functions on whole arrays of pairs, in the layout of
    raymond_sample_streams."""
    pairs = np.asarray(pairs, dtype=np.uint64).reshape(-1, 2)
    index, sample = pairs[:, 0], pairs[:, 1]
    sh = np.uint64(seed_hash)
    cols = []
    qmc_seed = u32(pcg(u32(index + np.uint64(0x9E3779B9))) ^ sh)
    for d in dim_ids:
        key = pcg(qmc_seed ^ pcg(np.full_like(index, d)))
        y = owen(sample, key)
        a = unit(owen(reverse_bits(y), pcg(key)))
        b = unit(owen(sobol2(y), pcg(u32(key + np.uint64(1)))))
        cols += [a, b, a]  # rand() at a dimension is rand2()'s first value
    spectrum = (u32(pcg(u32(index * np.uint64(7919) + np.uint64(1))) + u32(sample * np.uint64(2654435769)))
                >> np.uint64(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)
    cols.append(spectrum)
    for salt in (977, 4099):
        state = u32(pcg(index ^ pcg(u32(sample * np.uint64(2654435769) + np.uint64(salt)))) ^ sh)
        for _ in range(chain):
            state = pcg(state)
            cols.append(unit(state))
    return np.stack(cols, axis=1).astype(np.float32)


def cases():
    """Pixels across a 4K frame and sample indices from the first to ones
    whose Sobol index has its top bits set; dimensions of the lens, the first
    bounces' blocks ((depth + 1) << 16, :1271) and a few beyond."""
    rng = np.random.default_rng(5)
    pixels = np.concatenate([[0, 1, 2, 1023, 1024, 65535, 1048575, 3840 * 2160 - 1],
                             rng.integers(0, 3840 * 2160, 56)]).astype(np.uint64)
    samples = np.array([0, 1, 2, 3, 7, 8, 255, 256, 4095, 16383, 65536, 2 ** 24 + 3, 2 ** 31 - 1, 2 ** 31,
                        2 ** 32 - 1], dtype=np.uint64)
    pairs = np.stack(np.meshgrid(pixels, samples, indexing="ij"), axis=-1).reshape(-1, 2)
    dims = [0, 1, 2] + [((depth + 1) << 16) + k for depth in range(9) for k in (0, 1, 2, 3)] + [0xFFFFFFFF]
    return pairs.astype(np.uint32), np.array(dims, dtype=np.uint32)


@pytest.mark.parametrize("seed_hash", [0, 0x2545F491])
def test_oracle_streams_equal_the_shaders(seed_hash):
    """seed_hash 0 gives the reference's streams; another value (the
    renderer's per-instance seed) is XORed into every seed."""
    pairs, dims = cases()
    got = oracle.sample_streams(pairs, dims, 12, seed_hash)
    want = reference_streams(pairs, dims, 12, seed_hash)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_streams_are_uniform_and_distinct():
    pairs, dims = cases()
    s = oracle.sample_streams(pairs, dims, 12)
    assert (s >= 0).all() and (s < 1).all()
    assert len(np.unique(s[:, 0])) > 0.95 * len(s)


@pytest.mark.gpu
@pytest.mark.parametrize("seed_hash", [0, 0x2545F491])
def test_gpu_streams_equal_the_oracles_bit_for_bit(gpu, seed_hash):
    from raymond_gb300 import Canvas, Renderer, _native

    pairs, dims = cases()
    chain = 12
    r = Renderer.create(Canvas(8, 8))
    out = np.zeros((len(pairs), 3 * len(dims) + 1 + 2 * chain), dtype=np.float32)
    _native.check(_native.lib().raymond_sample_streams(r.handle, _native.ptr(pairs), len(pairs), _native.ptr(dims),
                                                       len(dims), chain, seed_hash, _native.ptr(out)), r.handle)
    r.dispose()
    want = oracle.sample_streams(pairs, dims, chain, seed_hash)
    diff = np.nonzero(out.view(np.uint32) != want.view(np.uint32))
    assert diff[0].size == 0, (diff[0][:5], diff[1][:5])
