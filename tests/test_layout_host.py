"""Host checks of the spectral layouts (no GPU): the index maps the kernels
and the conversions share are permutations of a solve's plane, and the
column pass's per-thread address arithmetic lands on them.

A small host program is compiled with nvcc against csrc/ptf_passes.cuh and
checks, for every line length, row grouping and column-group width the
library uses:

* spec_map (interleaved rows, register order, 3D planes) maps the
  rows x pitch elements of a solve one-to-one onto [0, rows * pitch);
* the column pass's offsets -- tb + (row offset) * stride for the
  interleaved layout, pb + i * (TPL << pl) for register order, with
  tb, pb as the kernel forms them -- equal spec_index / priv_index of the
  position the thread holds (reg_pos of the last forward stage);
* the two rows of a row pair are adjacent when rows are interleaved.
"""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parents[1] / "passivetracerflows.jl_gb300" / "csrc"

PROGRAM = r"""
#include <cstdio>
#include <vector>
#include "ptf_passes.cuh"
using namespace ptf;

static int fails = 0;
#define CHECK(c, ...) do { if (!(c)) { if (fails++ < 10) { std::printf(__VA_ARGS__); std::printf("\n"); } } } while (0)

template <int N> void check_len() {
  typedef float T;
  constexpr int E = ColE<T, N>::value, TPL = col_tpl<T, N>(), RF = LastRadix<N, -1, E>::value;
  for (int pl = 1; pl <= 2; ++pl)
    for (int yl = 0; yl <= col_ylog_max<T, N>(); ++yl)
      for (int pitch : {8, 16, 24, 40, 72, 136, 264, 520}) {
        // 2D: rows = N along the column pass
        SpecMap m; m.pitch = pitch; m.ylog = yl; m.n = N; m.tpl = TPL; m.rf = RF; m.pl = pl;
        for (int priv = 0; priv <= 1; ++priv) {
          m.priv = priv;
          std::vector<char> seen((size_t)N * pitch, 0);
          for (int r = 0; r < N; ++r)
            for (int k = 0; k < pitch; ++k) {
              const long long x = spec_map(m, r, k);
              CHECK(x >= 0 && x < (long long)N * pitch, "N=%d out of range", N);
              if (x >= 0 && x < (long long)N * pitch) { CHECK(!seen[x], "N=%d priv=%d yl=%d: %lld twice", N, priv, yl, x); seen[x] = 1; }
            }
        }
        // the kernel's address arithmetic (col_body) for every thread and register
        const int stride = pitch, PLc = pl;
        for (int col = 0; col < pitch; ++col)
          for (int t = 0; t < TPL; ++t) {
            const int tb = (((t >> yl) * stride + col) << yl) + (t & ((1 << yl) - 1));
            const int pb = (((col >> PLc) * N + t) << PLc) + (col & ((1 << PLc) - 1));
            for (int i = 0; i < E; ++i) {
              const int p = t + (i / RF) * TPL + (i % RF) * (N / RF);  // reg_pos of the last forward stage
              const int off = tb + ((i / RF) * TPL + (i % RF) * (N / RF)) * stride;
              CHECK(off == spec_index(p, col, pitch, yl), "N=%d yl=%d col=%d t=%d i=%d: layout offset", N, yl, col, t, i);
              SpecMap mp = m; mp.priv = 1;
              CHECK(pb + i * (TPL << PLc) == priv_index(mp, p, col), "N=%d pl=%d col=%d t=%d i=%d: register order", N, pl, col, t, i);
            }
          }
        // row pairs are adjacent when rows are interleaved
        if (yl >= 1)
          for (int y0 = 0; y0 < N; y0 += 2)
            for (int k = 0; k < pitch; ++k) CHECK(spec_index(y0 + 1, k, pitch, yl) == spec_index(y0, k, pitch, yl) + 1, "pair");
      }
}

void check_3d() {
  // 3D: the main pass runs along z over planes of ny interleaved rows
  typedef float T;
  constexpr int NZ = 32, E = ColE<T, NZ>::value, TPL = col_tpl<T, NZ>(), RF = LastRadix<NZ, -1, E>::value;
  for (int ny : {16, 64}) {
    SpecMap m; m.pitch = 24; m.ylog = ny >= 64 ? 2 : 0; m.priv = 1; m.n = NZ; m.tpl = TPL; m.rf = RF; m.pl = 2;
    m.ny = ny; m.three = 1;
    const long long total = (long long)NZ * ny * m.pitch;
    std::vector<char> seen(total, 0);
    for (int r = 0; r < NZ * ny; ++r)
      for (int k = 0; k < m.pitch; ++k) {
        const long long x = spec_map(m, r, k);
        CHECK(x >= 0 && x < total && !seen[x], "3D ny=%d: not a permutation", ny);
        if (x >= 0 && x < total) seen[x] = 1;
      }
  }
}

int main() {
  check_len<16>(); check_len<32>(); check_len<64>(); check_len<128>(); check_len<256>(); check_len<512>();
  check_len<1024>();
  check_3d();
  std::printf(fails ? "FAIL %d\n" : "OK\n", fails);
  return fails ? 1 : 0;
}
"""


def test_layout_maps_and_kernel_offsets(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    src = tmp_path / "layout_check.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "layout_check"
    r = subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-O1", "-I", str(CSRC), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.strip().endswith("OK"), out.stdout + out.stderr
