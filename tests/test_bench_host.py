"""Host-side logic of bench.py, on the CPU: the algorithmic bytes of each
launch read from a plan's description (rows of its input and output views
at the element size of the buffer each lives in), the kernel named in the
roofline (register kernels, fused launches), and the DRAM traffic looked
up in the committed ncu summary."""

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


class FakePlan:
    """The two members of a plan that bench's accounting reads."""

    def __init__(self, compute_type, text):
        self.compute_type = compute_type
        self._text = text

    def describe(self, direction=0):
        return self._text


# the Kron workload's FP32 description: C and H fused, then F
KRON_FP32 = (
    "launch src=0 dst=1 in=(65536,128,1) out=(65536,128,1) rconv L=128 "
    "acc=0: fft-conv fused-with-next\n"
    "launch src=1 dst=1 in=(256,256,128) out=(256,256,128) rfwht L=256 "
    "stride=256 fused-with-previous acc=0: fwht(256)\n"
    "launch src=1 dst=1 in=(1,256,32768) out=(1,256,32768) rsfft L=256 "
    "stride=32768 acc=0: fft(256, sign -1)\n")

HADAMARD_FP32 = (
    "launch src=0 dst=1 in=(512,8192,1) out=(512,8192,1) rfwht L=8192 "
    "stride=1 fused-with-next acc=0: fwht(8192)\n"
    "launch src=1 dst=1 in=(1,512,8192) out=(1,512,8192) rfwht L=512 "
    "stride=8192 fused-with-previous acc=0: fwht(512)\n")


def test_launch_bytes_from_views():
    N, M = 1 << 23, 8
    plan = FakePlan(6, KRON_FP32)   # FM_C64
    lb = bench.launch_bytes(plan, N, N, M, 8, 8)
    # every launch streams each column once in and once out
    assert lb == [M * N * 16] * 3
    N2 = 1 << 22
    plan = FakePlan(4, HADAMARD_FP32)  # FM_F32
    assert bench.launch_bytes(plan, N2, N2, 64, 4, 4) == [64 * N2 * 8] * 2


def test_roofline_names_the_register_and_fused_kernels():
    import fastmat_gb300 as fg
    N, M = 1 << 23, 8
    # the fused launch takes the time, its partner line none
    r = bench.roofline_of(fg, FakePlan(6, KRON_FP32), [0.344, 0.002, 0.177],
                          N, N, M, np.complex64, np.complex64, 6800.3,
                          'measured', 'kron', 'fp32')
    assert r['kernel'].startswith('rkch') and r['kernel'].endswith('1 of 3')
    assert abs(r['achieved'] - M * N * 16 / 0.344e-3 / 1e9) < 1e-6
    assert abs(r['frac'] - r['achieved'] / 6800.3) < 1e-12
    r = bench.roofline_of(fg, FakePlan(6, KRON_FP32), [0.1, 0.0, 0.2],
                          N, N, M, np.complex64, np.complex64, 6800.3,
                          'measured', 'kron', 'fp32')
    assert r['kernel'] == 'rsfft launch 3 of 3'
    N2 = 1 << 22
    r = bench.roofline_of(fg, FakePlan(4, HADAMARD_FP32), [0.674, 0.002],
                          N2, N2, 64, np.float32, np.float32, 6800.3,
                          'measured', 'hadamard', 'fp32')
    assert r['kernel'].startswith('rfwht2')


def test_traffic_lookup_in_the_committed_summary():
    assert bench.ncu_traffic('kron', 'fp32', 1) is not None
    assert bench.ncu_traffic('kron', 'fp64', 3) is not None
    assert bench.ncu_traffic('hadamard', 'fp32', 1) is not None
    # a fused pair's second line launches nothing and has no entry
    assert bench.ncu_traffic('hadamard', 'fp32', 2) is None
    assert bench.ncu_traffic('nothing', 'fp32', 1) is None
