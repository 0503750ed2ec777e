"""Many solver domains stepped together (include/aeros_batch.h).

A Batch holds Solver objects of one storage type and advances all of them with
one persistent kernel per lattice step, a chunk of steps replayed as a CUDA
graph. Fields, forces and statistics are read through each member Solver, as
for a lone domain; a member gives the same bits alone as in any mix.
"""
from __future__ import annotations

import ctypes as C

from .capi import STORAGE_NAMES, BatchTuning, check, lib
from .solver import Solver


class Batch:
    def __init__(self, storage="fp16"):
        st = STORAGE_NAMES[storage] if isinstance(storage, str) else int(storage)
        h = C.c_void_p()
        check(lib().aeros_batch_create(st, C.byref(h)), "aeros_batch_create")
        self.h = h
        self.members: list[Solver] = []

    def close(self) -> None:
        if getattr(self, "h", None):
            lib().aeros_batch_destroy(self.h)
            self.h = None
            self.members = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def add(self, s: Solver) -> None:
        check(lib().aeros_batch_add(self.h, s.h), "aeros_batch_add")
        self.members.append(s)

    def remove(self, s: Solver) -> None:
        check(lib().aeros_batch_remove(self.h, s.h), "aeros_batch_remove")
        self.members.remove(s)

    def size(self) -> tuple[int, int]:
        n, c = C.c_int32(), C.c_int64()
        check(lib().aeros_batch_size(self.h, C.byref(n), C.byref(c)), "aeros_batch_size")
        return int(n.value), int(c.value)

    def step(self, n: int) -> None:
        check(lib().aeros_batch_step(self.h, int(n)), "aeros_batch_step")

    @property
    def tuning(self) -> dict:
        t = BatchTuning()
        check(lib().aeros_batch_get_tuning(self.h, C.byref(t)), "aeros_batch_get_tuning")
        return t.as_dict()

    def set_tuning(self, blocks_per_sm=0, tiles_per_item=1, shell_tiles_per_item=1, chunk_steps=20) -> None:
        t = BatchTuning()
        t.blocks_per_sm, t.tiles_per_item = int(blocks_per_sm), int(tiles_per_item)
        t.shell_tiles_per_item, t.chunk_steps = int(shell_tiles_per_item), int(chunk_steps)
        check(lib().aeros_batch_set_tuning(self.h, C.byref(t)), "aeros_batch_set_tuning")

    def autotune(self, trial_steps: int = 20) -> dict:
        t = BatchTuning()
        check(lib().aeros_batch_autotune(self.h, int(trial_steps), C.byref(t)), "aeros_batch_autotune")
        return t.as_dict()

    def last_step_ms(self) -> float:
        v = C.c_float()
        check(lib().aeros_batch_last_step_ms(self.h, C.byref(v)), "aeros_batch_last_step_ms")
        return float(v.value)

    def last_launch_count(self) -> int:
        v = C.c_int64()
        check(lib().aeros_batch_last_launch_count(self.h, C.byref(v)), "aeros_batch_last_launch_count")
        return int(v.value)
