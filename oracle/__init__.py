"""CPU oracle for adaptive RBRP column ID (test infrastructure only).

This package is the parity checker for the CUDA path.  Only the test suite,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference`` legs
of ``bench.py`` may import it, and only as the checker or as the timed CPU
baseline: the product path never routes through it.

Parity is pinned against the reference's own Python RBRP
(``python/RBRP.ipynb`` cells 2, 7, 11), run in the development container to
produce the fixtures under ``tests/golden/`` (see ``tests/golden/make_golden.py``).
"""
from .philox import philox4x64_10, PhiloxStream, es_uniforms
from .rbrp_oracle import (
    np_compat_choice,
    es_topb,
    local_clip,
    corrected_swap,
    rbrp_column_id,
    interp_sid,
    interp_r11,
    id_error,
    error_at_rank,
    matdivide,
)

__all__ = [
    "philox4x64_10",
    "PhiloxStream",
    "es_uniforms",
    "np_compat_choice",
    "es_topb",
    "local_clip",
    "corrected_swap",
    "rbrp_column_id",
    "interp_sid",
    "interp_r11",
    "id_error",
    "error_at_rank",
    "matdivide",
]
