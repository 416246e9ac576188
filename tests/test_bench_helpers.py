"""Host-side helpers of bench.py that shape its JSON line: the names of the
batched launches the roofline is taken over, and the algorithmic bytes of
each kernel of the 4K 4:2:2 workload."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "svt-jpeg-xs_gb300"))

import bench  # noqa: E402
import jxs  # noqa: E402


def test_launch_names_cover_the_kernel_table():
    """Every stage the library's stage timing reports maps to one of the
    bench's kernel names; transform levels by their variant (0: the 32-bit
    low band of the deeper level)."""
    names = {bench.launch_name(s, v) for s in jxs.Batch.STAGES for v in (0, 2)}
    assert names == set(bench.ENC_KERNELS) | set(bench.DEC_KERNELS)
    assert bench.launch_name("fwd_v", 2) == "fwd_v_level0" and bench.launch_name("fwd_v", 0) == "fwd_v_level1"
    assert bench.launch_name("inv_v", 1) == "inv_v_level0" and bench.launch_name("inv_v", 0) == "inv_v_level1"
    assert bench.launch_name("rc", 0) == "rc_cost"


def test_kernel_bytes_of_the_4k_stream():
    """Compulsory bytes per frame: 16.6 M samples of 2 bytes in and out; the
    transform's first level reads them once, the inverse's writes them once;
    packing reads the coefficients and GCLIs and writes the codestream."""
    lcod = bench.W * bench.H * bench.BPP // 8
    kb = bench.kernel_bytes(lcod)
    samples = bench.W * bench.H * 2
    assert set(kb) == (set(bench.ENC_KERNELS) | set(bench.DEC_KERNELS)) - {"walk"}
    assert kb["pack"] == 2 * samples + samples // 4 + lcod
    assert kb["unpack"] == lcod + 2 * samples
    assert kb["fwd_v_level0"] > 2 * samples and kb["inv_v_level0"] > 2 * samples
    assert kb["rc_cost"] == samples // 4
    # every kernel with DRAM traffic recorded has algorithmic bytes
    assert set(bench.KERNEL_DRAM_BYTES) <= set(kb)
