"""Host-side checks of the walk-on-stars and batched-mesh plumbing: the ctypes
mirrors of snch_wost_params / snch_wost_stats have the C header's layout
(compiled and measured with the host C compiler), and the batched workload
generator is deterministic with log-uniform triangle counts."""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_wost_struct_layout_matches_header(tmp_path):
    from snch_lbvh_gb300.wost import MAX_STEPS, WostParams, WostStats
    src = tmp_path / "layout.c"
    src.write_text(r"""
#include <stddef.h>
#include <stdio.h>
#include "snch_gb300.h"
int main(void) {
  printf("%d %zu %zu %zu %zu %zu %zu %zu %zu\n", SNCH_WOST_MAX_STEPS, sizeof(snch_wost_params),
         offsetof(snch_wost_params, max_steps), offsetof(snch_wost_params, center), offsetof(snch_wost_params, seed),
         offsetof(snch_wost_params, floor_), sizeof(snch_wost_stats), offsetof(snch_wost_stats, step_ms),
         offsetof(snch_wost_stats, fallback));
  return 0;
}
""")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c11", str(src), "-I", os.path.join(ROOT, "include"), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [MAX_STEPS, C.sizeof(WostParams), WostParams.max_steps.offset, WostParams.center.offset,
            WostParams.seed.offset, WostParams.floor_.offset, C.sizeof(WostStats), WostStats.step_ms.offset,
            WostStats.fallback.offset]
    assert got == want


def test_batched_meshes_generator():
    from snch_lbvh_gb300 import meshes
    a = meshes.batched_meshes(seed=3, count=12, lo=200, hi=5000)
    b = meshes.batched_meshes(seed=3, count=12, lo=200, hi=5000)
    assert len(a) == 12
    for (va, fa), (vb, fb) in zip(a, b):
        np.testing.assert_array_equal(va, vb)
        np.testing.assert_array_equal(fa, fb)
        assert va.dtype == np.float32 and fa.dtype == np.int32
        assert fa.min() >= 0 and fa.max() < len(va)
        c = 0.5 * (va.min(0) + va.max(0))
        assert np.all((c >= 0) & (c <= 1))  # placed in the unit cube (centred there when wider)
    counts = [len(f) for _, f in a]
    assert min(counts) >= 80 and max(counts) <= 4 * 5000
