"""The tile-major layout of the packed signals (cdm_tile_index /
cdm_tile_elems in csrc/kernels/cdm_args.h), checked on the host: every
(voxel, row, lane) of a pack lands on its own element inside the allocated
whole tiles, a lane's next row is CDM_NT elements on, and a CTA's voxels
own one contiguous block. Compiled with nvcc as host code for the default
CTA size and the 64- and 256-thread build variants."""
import os
import subprocess

import pytest

from cudimot_gb300 import build

SRC = r"""
#define NPARAMS 5
#define CDM_PSTORE 5
#define CDM_CFP_TSIZE 4
#define CDM_FIXP_TSIZE 1
#define CDM_NDCFP 0
#include "cdm_args.h"
#include <cstdio>
#include <vector>

int main() {
  const int lanes[] = {1, 2, 4, 8, 16, 32};
  const int nvoxs[] = {1, 2, 31, 32, 63, 64, 65, 127, 1000, 4097};
  const int rowss[] = {1, 2, 37, 74, 144};
  for (int Gw : lanes)
    for (int nvox : nvoxs)
      for (int rows : rowss) {
        const size_t n = cdm_tile_elems(nvox, rows, Gw);
        std::vector<unsigned char> seen(n, 0);
        const int vpt = CDM_NT / Gw;
        for (int v = 0; v < nvox; v++)
          for (int r = 0; r < rows; r++)
            for (int j = 0; j < Gw; j++) {
              const size_t i = cdm_tile_index(v, r, j, rows, Gw);
              if (i >= n || seen[i]) {
                printf("bad G=%d nvox=%d rows=%d v=%d r=%d j=%d i=%zu n=%zu\n", Gw, nvox, rows, v,
                       r, j, i, n);
                return 1;
              }
              seen[i] = 1;
              if (r + 1 < rows && cdm_tile_index(v, r + 1, j, rows, Gw) != i + CDM_NT) {
                printf("stride G=%d rows=%d\n", Gw, rows);
                return 1;
              }
              // the tile's block: [tile * rows * CDM_NT, (tile + 1) * rows * CDM_NT)
              const size_t t = (size_t)(v / vpt);
              if (i < t * rows * CDM_NT || i >= (t + 1) * rows * CDM_NT) {
                printf("block G=%d nvox=%d rows=%d v=%d\n", Gw, nvox, rows, v);
                return 1;
              }
            }
        // whole tiles, nothing more
        const size_t tiles = ((size_t)nvox + vpt - 1) / vpt;
        if (n != tiles * rows * CDM_NT) {
          printf("size G=%d nvox=%d rows=%d\n", Gw, nvox, rows);
          return 1;
        }
      }
  printf("ok\n");
  return 0;
}
"""


@pytest.mark.parametrize("nt", [128, 64, 256])
def test_tile_layout(tmp_path, nt):
    src = tmp_path / "tile.cu"
    src.write_text(SRC)
    exe = tmp_path / "tile"
    kdir = os.path.join(build.CSRC, "kernels")
    r = subprocess.run([build.nvcc_path(), "-std=c++17", f"-DCDM_NT={nt}", "-I", kdir, str(src),
                        "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout + out.stderr
