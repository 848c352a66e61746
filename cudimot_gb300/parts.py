"""Voxel partitioning, as CUDIMOT splits a volume.

shard_range: the job-level split of split_parts.cc:80-94 (--nParts): every
part has nvox // nparts voxels and the last part takes the remainder. Used
to give each GPU/rank its own contiguous voxel range; voxels are
independent, so the fit needs no communication between ranks.

subparts: the in-process split of dMRI_Data.cu:65-79 (SIZE_PART = 12800);
a last part smaller than half a part is spread over the others.
"""
from __future__ import annotations

SIZE_PART = 12800


def shard_range(nvox: int, nparts: int, idpart: int) -> tuple[int, int]:
    if nparts <= 0 or not (0 <= idpart < nparts):
        raise ValueError("idpart must be in [0, nparts)")
    if nvox < nparts:
        raise ValueError("the number of parts must not exceed the number of voxels")
    size = nvox // nparts
    start = idpart * size
    stop = nvox if idpart == nparts - 1 else start + size
    return start, stop


def subparts(nvox: int, size_part: int = SIZE_PART) -> list[tuple[int, int]]:
    if nvox <= 0:
        return []
    nparts = nvox // size_part + (1 if nvox % size_part else 0)
    size = size_part
    last = nvox - (nparts - 1) * size
    if last < size_part * 0.5:
        if nparts - 1:
            size = size + last // (nparts - 1)
            nparts -= 1
        else:
            size = 0
    out = []
    for i in range(nparts):
        a = i * size
        b = nvox if i == nparts - 1 else a + size
        out.append((a, b))
    return out
