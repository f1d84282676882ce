"""Host allocation failure through the DN_set_allocator hook (no GPU needed).

The reference allocates through DN_MALLOC / DN_REALLOC / DN_FREE (globals.h) and reports failures with a
NULL / false return plus an error message.  Here an allocator that fails after n calls is installed and
every n is tried for a CPU-only volume with edits: each attempt must fail cleanly (NULL, or false with an
error message) or succeed, never crash, and the volume must stay usable or be NULL.
"""
import ctypes
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import doonengine_gb300 as dn          # noqa: E402
from doonengine_gb300 import _lib as L  # noqa: E402

libc = ctypes.CDLL(None)
libc.malloc.restype = ctypes.c_void_p
libc.malloc.argtypes = [ctypes.c_size_t]
libc.realloc.restype = ctypes.c_void_p
libc.realloc.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
libc.free.argtypes = [ctypes.c_void_p]

MALLOC = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_size_t)
FREE = ctypes.CFUNCTYPE(None, ctypes.c_void_p)
REALLOC = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t)


class FailingAllocator:
    def __init__(self, budget):
        self.budget = budget
        self.calls = 0
        self.m = MALLOC(self._malloc)
        self.f = FREE(lambda p: libc.free(p))
        self.r = REALLOC(self._realloc)

    def _malloc(self, n):
        self.calls += 1
        return None if self.calls > self.budget else libc.malloc(n)

    def _realloc(self, p, n):
        self.calls += 1
        return None if self.calls > self.budget else libc.realloc(p, n)


def test_allocation_failures_are_reported_not_fatal():
    lib = L.load()
    lib.DN_set_allocator.argtypes = [MALLOC, FREE, REALLOC]
    dn.install_message_callback()
    errors_before = len(dn.messages())
    outcomes = {"null": 0, "ok": 0}
    try:
        for budget in range(0, 40):
            alloc = FailingAllocator(budget)
            lib.DN_set_allocator(alloc.m, alloc.f, alloc.r)
            ptr = lib.DN_create_volume_cpu(L.DNuvec3(4, 4, 4), 8)
            if not ptr:
                outcomes["null"] += 1
                continue
            vol = dn.Volume(None, _ptr=ptr)
            # edits that need new chunks (and more chunk memory) past the allocation budget
            for i in range(12):
                vol.set_voxel((i % 4, (i // 4) % 4, i // 16), (1, 2, 3), 1, (0.0, 1.0, 0.0), (10, 20, 30))
            outcomes["ok"] += 1
            vol.close()
    finally:
        lib.DN_set_allocator(ctypes.cast(None, MALLOC), ctypes.cast(None, FREE), ctypes.cast(None, REALLOC))
    assert outcomes["null"] > 0 and outcomes["ok"] > 0, outcomes
    # every refused allocation surfaced as a message
    assert len(dn.messages()) > errors_before
