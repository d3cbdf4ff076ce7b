"""JSSP instances: the reference's text format, path resolution, synthetic generation.

Mirrors cpu/common/instance_parser.cpp (``resolve_instance_file`` :8-34,
``parse_instance`` :37-93) and the ``Operation`` / ``JSSPInstance`` types of
cpu/common/jssp_types.h:8-23, so that a file the reference reads gives the same
instance here.  The synthetic generator writes that same text format, so the
reference and this library parse identical bytes.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

__all__ = [
    "Operation",
    "JSSPInstance",
    "parse_instance",
    "resolve_instance_file",
    "format_instance",
    "write_instance",
    "synthetic_instance",
    "schedule_makespan",
]

_MASK64 = (1 << 64) - 1


@dataclass
class Operation:
    """One operation (cpu/common/jssp_types.h:8-13): 1-based op, machine and job ids."""

    num_op: int
    num_mc: int
    dure: int
    num_j: int


@dataclass
class JSSPInstance:
    """Problem instance (cpu/common/jssp_types.h:16-23).

    ``operations`` holds ``nboperation = nbjob*nbmachine + 2`` entries: a dummy op 0,
    the real ops ``j*m + k + 1`` in job order, and a dummy op ``n*m + 1``; machines are
    1-based (instance_parser.cpp:51-83).  ``machine`` / ``duration`` are the compact
    0-based ``[n, m]`` arrays the solver library takes.
    """

    nbjob: int = 0
    nbmachine: int = 0
    nboperation: int = 0
    operations: List[Operation] = field(default_factory=list)
    opr_mach: List[List[int]] = field(default_factory=list)

    @property
    def machine(self) -> np.ndarray:
        n, m = self.nbjob, self.nbmachine
        a = np.array([op.num_mc - 1 for op in self.operations[1 : n * m + 1]], dtype=np.int32)
        return a.reshape(n, m)

    @property
    def duration(self) -> np.ndarray:
        n, m = self.nbjob, self.nbmachine
        a = np.array([op.dure for op in self.operations[1 : n * m + 1]], dtype=np.int32)
        return a.reshape(n, m)

    @classmethod
    def from_arrays(cls, machine: Sequence[Sequence[int]], duration: Sequence[Sequence[int]]) -> "JSSPInstance":
        mc = np.asarray(machine, dtype=np.int64)
        du = np.asarray(duration, dtype=np.int64)
        if mc.ndim != 2 or mc.shape != du.shape:
            raise ValueError("machine and duration must be [n, m] arrays of the same shape")
        n, m = mc.shape
        inst = cls(nbjob=int(n), nbmachine=int(m), nboperation=int(n * m + 2))
        inst.operations.append(Operation(0, 0, 0, 0))
        inst.opr_mach = [[] for _ in range(m + 1)]
        idf = 1
        for j in range(n):
            for k in range(m):
                inst.operations.append(Operation(idf, int(mc[j, k]) + 1, int(du[j, k]), j + 1))
                if 0 <= mc[j, k] < m:
                    inst.opr_mach[int(mc[j, k]) + 1].append(idf)
                idf += 1
        inst.operations.append(Operation(n * m + 1, 0, 0, 0))
        return inst


def resolve_instance_file(input_arg: str) -> Optional[str]:
    """Resolve a path or benchmark id the way instance_parser.cpp:8-34 does.

    The argument is first tried as a path, then through the reference's list of
    formats (Lawrence first; Taillard ids without a ``.txt`` suffix).  Returns the
    first existing path or ``None``.
    """
    if os.path.isfile(input_arg):
        return input_arg
    formats = (
        "./la%s.txt",
        "./ta%s.txt",
        "./lawrence_instances/la%s.txt",
        "../lawrence_instances/la%s.txt",
        "../../lawrence_instances/la%s.txt",
        "./taillard_instances/ta%s",
        "../taillard_instances/ta%s",
        "../../taillard_instances/ta%s",
    )
    for fmt in formats:
        cand = fmt % input_arg
        if os.path.isfile(cand):
            return cand
    return None


def _ints(text: str):
    """Yield successive integers as fscanf("%d") would, stopping at the first token
    that is not an integer (fscanf then keeps failing at the same place)."""
    for tok in text.split():
        try:
            yield int(tok, 10)
        except ValueError:
            return


def parse_instance(filepath: str) -> Optional[JSSPInstance]:
    """Parse an instance file (instance_parser.cpp:37-93).

    Returns ``None`` where the reference returns false (file cannot be opened, header
    unreadable).  Like the reference, values missing from a truncated body read as
    machine 0 / duration 0.
    """
    try:
        with open(filepath, "r") as f:
            text = f.read()
    except OSError:
        return None
    it = _ints(text)
    try:
        n = next(it)
        m = next(it)
    except StopIteration:
        return None
    inst = JSSPInstance(nbjob=n, nbmachine=m, nboperation=n * m + 2)
    inst.operations.append(Operation(0, 0, 0, 0))
    inst.opr_mach = [[] for _ in range(max(m, 0) + 1)]
    idf = 1
    exhausted = False
    for job in range(1, n + 1):
        for _step in range(1, m + 1):
            mc = dur = 0
            if not exhausted:
                try:
                    mc = next(it)
                    dur = next(it)
                except StopIteration:
                    exhausted = True
            inst.operations.append(Operation(idf, mc + 1, dur, job))
            if 0 <= mc + 1 <= m:
                inst.opr_mach[mc + 1].append(idf)
            idf += 1
    inst.operations.append(Operation(n * m + 1, 0, 0, 0))
    return inst


def format_instance(machine: np.ndarray, duration: np.ndarray) -> str:
    """Text in the reference format: ``n m`` then one line per job of
    ``machine duration`` pairs (machines 0-based)."""
    n, m = machine.shape
    lines = [f"{n} {m}"]
    for j in range(n):
        lines.append(" ".join(f"{int(machine[j, k])} {int(duration[j, k])}" for k in range(m)))
    return "\n".join(lines) + "\n"


def write_instance(path: str, machine: np.ndarray, duration: np.ndarray) -> None:
    with open(path, "w") as f:
        f.write(format_instance(machine, duration))


class _SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & _MASK64

    def next(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
        return z ^ (z >> 31)

    def bounded(self, k: int) -> int:
        """Uniform integer in [0, k) by multiply-shift of the high 32 bits."""
        return ((self.next() >> 32) * k) >> 32


def synthetic_instance(n: int, m: int, seed: int, dmin: int = 1, dmax: int = 99):
    """Seeded synthetic instance with the shape of the Lawrence/Taillard families.

    splitmix64 stream seeded by ``seed``; for each job in order: a Fisher-Yates
    permutation of machines ``0..m-1`` (i = m-1 down to 1, swap with ``bounded(i+1)``),
    then ``m`` durations ``dmin + bounded(dmax-dmin+1)``.  Returns ``(machine,
    duration)`` as int32 ``[n, m]`` arrays.
    """
    rng = _SplitMix64(seed)
    machine = np.zeros((n, m), dtype=np.int32)
    duration = np.zeros((n, m), dtype=np.int32)
    span = dmax - dmin + 1
    for j in range(n):
        perm = list(range(m))
        for i in range(m - 1, 0, -1):
            r = rng.bounded(i + 1)
            perm[i], perm[r] = perm[r], perm[i]
        machine[j, :] = perm
        for k in range(m):
            duration[j, k] = dmin + rng.bounded(span)
    return machine, duration


def schedule_makespan(machine: np.ndarray, duration: np.ndarray, seq: Sequence[int]) -> int:
    """Makespan of a schedule given as 1-based op ids in dispatch order; -1 if the
    sequence is not a permutation that respects every job's operation order."""
    n, m = machine.shape
    tr = [0] * m
    jr = [0] * n
    nx = [0] * n
    cmax = 0
    if len(seq) != n * m:
        return -1
    for op in seq:
        op = int(op)
        if op < 1 or op > n * m:
            return -1
        j, k = divmod(op - 1, m)
        if k != nx[j]:
            return -1
        mc = int(machine[j, k])
        fin = max(tr[mc], jr[j]) + int(duration[j, k])
        tr[mc] = fin
        jr[j] = fin
        nx[j] += 1
        cmax = max(cmax, fin)
    return cmax
