"""CPU: the packed host layout of the batched form and the host-side argument checks of
HostBatch and of Batch over host-resident matrices."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_packed_offsets_align_every_matrix_to_16_bytes():
    from robust_blockwise_random_pivoting_gb300.rbrp import packed_offsets
    shapes = [(3, 5), (64, 64), (7, 1), (1, 1), (129, 33)]
    offs, sizes = packed_offsets(shapes)
    assert sizes.tolist() == [15, 4096, 7, 1, 4257]
    assert offs[0] == 0 and len(offs) == len(shapes) + 1
    assert all(o % 4 == 0 for o in offs)                        # 16-byte starts for FP32
    assert all(offs[q + 1] - offs[q] >= sizes[q] for q in range(len(shapes)))
    assert all(offs[q + 1] - offs[q] - sizes[q] < 4 for q in range(len(shapes)))


def test_host_batch_rejects_unpinned_or_misshaped_buffers():
    from robust_blockwise_random_pivoting_gb300.rbrp import HostBatch, packed_offsets
    shapes = [(8, 8), (5, 3)]
    offs, _ = packed_offsets(shapes)
    with pytest.raises(TypeError):
        HostBatch(torch.zeros(int(offs[-1]), dtype=torch.float32), shapes)          # not pinned
    with pytest.raises(TypeError):
        HostBatch(torch.zeros(int(offs[-1]), dtype=torch.float64), shapes)          # not FP32


def test_host_resident_batch_rejects_pageable_or_non_fp32_matrices():
    """Batch over host matrices wants FP32 views of pinned memory (checked before any library call)."""
    import types
    from robust_blockwise_random_pivoting_gb300.rbrp import Batch
    fake = types.SimpleNamespace(lib=None, device=0)
    with pytest.raises(TypeError):
        Batch(fake, [torch.zeros(4, 4).t()])                       # pageable
    with pytest.raises(TypeError):
        Batch(fake, [torch.zeros(4, 4, dtype=torch.float64).t()])  # not FP32
    with pytest.raises(ValueError):
        Batch(fake, [])
