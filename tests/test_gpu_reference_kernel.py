"""The reference's own GPU kernel on the same GB300.

oracle/_ref/ref_gpu.cubin is dynamicsGradientKernel
(helpers_GPU/dynamicsGradient.cuh:1257-1292) compiled unmodified for sm_103a,
and oracle/_ref/ref_const.bin its model constants from the reference's own
initTransforms / initInertiaTensors (oracle/Makefile builds both where the
reference tree is present; both are device code or data, so they run on a GPU
box of any host architecture).  The module is loaded through the CUDA driver
API into torch's context and launched as time_GPU.cu:326 launches it,
<<<N, dim3(32, 7)>>>, on [q | qd | u | qdd | Minv] per knot (time_GPU.cu:
137-158), with q̈ and dense Minv taken from the engine (the reference computes
them on the host first, :134).

Two launch shapes.  The reference checks its kernels with one thread per
block, dim3(1, 1) (time_GPU.cu:9-10, TEST_FOR_EQUIVALENCE), and times them with
dim3(32, NUM_POS) (:12-18).  In the timed shape the kernel's results are wrong:
updateTransforms_GPU copies the top-left 3x3 block of each joint transform to
the bottom-right with a loop that starts every thread at index 0 instead of its
own (helpers_GPU/dynamicsGradient.cuh:406-410, kcr = 0 with kcr += delta), so
with 224 threads only the first of the 63 entries is copied and the others keep
the q-independent values of initTransforms.  With one thread the loop covers
them all.

Checked: in the one-thread shape the reference kernel and the engine both meet
the parity bar against the FP64 oracle, and agree with each other; in the
timed shape the reference kernel misses it, as the loop above says.  Timed
(printed with -s): one launch of the engine and of the reference kernel in both
shapes at the reference's batch sizes, its "Completely Fused - GPU Compute" row
(time_GPU.cu:322-330).  The engine's launch also produces q̈ and Minv, which the
reference kernel takes as inputs.
"""
import ctypes
import json
import os

import numpy as np
import pytest
import torch

import frg
import frg_oracle

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CUBIN = os.path.join(REPO, "oracle", "_ref", "ref_gpu.cubin")
CONST = os.path.join(REPO, "oracle", "_ref", "ref_const.bin")
NJ = 7
TOL = 1e-4  # max Frobenius-relative error of a knot's gradient


def _require_module():
    if not (os.path.exists(CUBIN) and os.path.exists(CONST)):
        pytest.skip("oracle/_ref holds no build of the reference's GPU kernel (built only where the "
                    "reference tree is present)")


class RefModule:
    """The cubin's kernels, by template arguments (KNOT_POINTS, MPC_MODE, VEL_DAMPING)."""

    def __init__(self):
        torch.zeros(1, device="cuda")  # torch's primary context is current on this thread
        cu = ctypes.CDLL("libcuda.so.1")
        self.cu = cu
        self.mod = ctypes.c_void_p()
        self._ok(cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        count = ctypes.c_uint()
        self._ok(cu.cuModuleGetFunctionCount(ctypes.byref(count), self.mod), "cuModuleGetFunctionCount")
        funcs = (ctypes.c_void_p * count.value)()
        self._ok(cu.cuModuleEnumerateFunctions(funcs, count, self.mod), "cuModuleEnumerateFunctions")
        cu.cuFuncGetName.argtypes = [ctypes.POINTER(ctypes.c_char_p), ctypes.c_void_p]
        self.by_name = {}
        for f in funcs:
            name = ctypes.c_char_p()
            self._ok(cu.cuFuncGetName(ctypes.byref(name), f), "cuFuncGetName")
            self.by_name[name.value.decode()] = f
        cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                                 ctypes.c_void_p, ctypes.c_void_p]

    def _ok(self, r, what):
        assert r == 0, f"{what}: CUresult {r}"

    def kernel(self, knots, mpc, damping):
        # Itanium mangling of dynamicsGradientKernel<float, knots, mpc, damping>
        prefix = f"_Z22dynamicsGradientKernelIfLi{knots}ELb{int(mpc)}ELb{int(damping)}EE"
        hits = [f for n, f in self.by_name.items() if n.startswith(prefix)]
        assert len(hits) == 1, f"{prefix} not in {sorted(self.by_name)}"
        return hits[0]

    def launch(self, f, knots, dqdd, mem_vol, mem_const, stream, block=(32, NJ)):
        args = [ctypes.c_void_p(t.data_ptr()) for t in (dqdd, mem_vol, mem_const)]
        params = (ctypes.c_void_p * 3)(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
        self._ok(self.cu.cuLaunchKernel(f, knots, 1, 1, block[0], block[1], 1, 0, ctypes.c_void_p(stream.cuda_stream),
                                        params, None), "cuLaunchKernel")

    def close(self):
        self.cu.cuModuleUnload(self.mod)


@pytest.fixture(scope="module")
def ref():
    _require_module()
    m = RefModule()
    yield m
    m.close()


def _case(ctx, n, seed):
    """Engine results on n knots and the reference kernel's inputs for them."""
    q, qd, u = (torch.from_numpy(x).cuda() for x in frg.sample_knots(n, seed=seed))
    dqdd = torch.empty((n, 2 * NJ * NJ), device="cuda")
    qdd = torch.empty((n, NJ), device="cuda")
    minv = torch.empty((n, NJ * NJ), device="cuda")
    ctx.gradient(n, q, qd, u, dqdd, qdd, minv)
    torch.cuda.synchronize()
    mem_vol = torch.cat([q, qd, u, qdd, minv], dim=1).contiguous()  # [q | qd | u | qdd | Minv]
    return (q, qd, u), (dqdd, qdd, minv), mem_vol


def _frob_rel(a, b):
    a = a.double()
    b = b.double()
    return ((a - b).norm(dim=1) / b.norm(dim=1).clamp_min(1e-30)).cpu().numpy()


@pytest.mark.parametrize("mpc,damping", [(False, False), (False, True), (True, False), (True, True)])
def test_engine_matches_reference_gpu_kernel(ref, mpc, damping):
    n = 1024
    const = torch.from_numpy(np.fromfile(CONST, np.float32)).cuda()
    assert const.numel() == 72 * NJ
    with frg.Context(vel_damping=damping, mpc_mode=mpc) as ctx:
        (q, qd, u), (dqdd, qdd, minv), mem_vol = _case(ctx, n, seed=900 + 2 * mpc + damping)
        f = ref.kernel(n, mpc, damping)
        out = torch.full((n, 2 * NJ * NJ), float("nan"), device="cuda")
        ref.launch(f, n, out, mem_vol, const, torch.cuda.current_stream(), block=(1, 1))
        timed_shape = torch.full((n, 2 * NJ * NJ), float("nan"), device="cuda")
        ref.launch(f, n, timed_shape, mem_vol, const, torch.cuda.current_stream())
        torch.cuda.synchronize()
    assert torch.isfinite(out).all()
    rd, _, _ = frg_oracle.gradient_f64(q.cpu().numpy(), qd.cpu().numpy(), u.cpu().numpy(), damping=damping, mpc=mpc)
    rd = torch.from_numpy(rd)
    e_engine = _frob_rel(dqdd.cpu(), rd)
    e_ref = _frob_rel(out.cpu(), rd)
    e_pair = _frob_rel(dqdd.cpu(), out.cpu())
    e_timed = _frob_rel(timed_shape.cpu(), rd)
    print(f"\nmpc={mpc} damping={damping}: max Frobenius-relative error vs FP64: engine {e_engine.max():.2e}, "
          f"reference GPU kernel {e_ref.max():.2e} with dim3(1,1); engine vs reference kernel {e_pair.max():.2e}; "
          f"reference kernel with dim3(32,7): median {np.median(e_timed):.2e}, "
          f"{(e_timed > TOL).mean() * 100:.1f} % of knots over the bar")
    assert e_engine.max() <= TOL
    assert e_ref.max() <= TOL
    assert e_pair.max() <= 2 * TOL
    assert (e_timed > TOL).mean() > 0.5  # the transform-copy loop of the timed shape (module docstring)


def _time_us(fn, stream, reps=20):
    for _ in range(3):
        fn()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) * 1e3 / reps


def test_time_reference_gpu_kernel_beside_engine(ref):
    """One launch of each at the reference's batch sizes (time_GPU.cu's main),
    CUDA events on one stream, 3 warm-up and 20 timed launches back to back
    (inputs of 20 MB at most, so L2-resident for both); the engine autotuned for
    each size, as a user would.  The reference kernel in its timed shape
    dim3(32, 7) and in its one-thread checking shape dim3(1, 1), whose results
    are the correct ones (module docstring); the one-thread shape is timed up to
    1,024 knots (one CTA per knot; at 65,536 knots a launch takes seconds)."""
    const = torch.from_numpy(np.fromfile(CONST, np.float32)).cuda()
    stream = torch.cuda.current_stream()
    rows = []
    for n in (16, 32, 64, 128, 1024, 65536):
        with frg.Context() as ctx:
            ctx.autotune(max(n, 32))  # the autotuner times batches of at least one tile
            (q, qd, u), (dqdd, qdd, minv), mem_vol = _case(ctx, n, seed=n)
            out = torch.empty((n, 2 * NJ * NJ), device="cuda")
            f = ref.kernel(n, False, False)
            t_ref = _time_us(lambda: ref.launch(f, n, out, mem_vol, const, stream), stream)
            t_one = None
            if n <= 1024:
                t_one = _time_us(lambda: ref.launch(f, n, out, mem_vol, const, stream, block=(1, 1)), stream, reps=3)
                err = float(_frob_rel(dqdd.cpu(), out.cpu()).max())
                assert err <= 2 * TOL
            t_eng = _time_us(lambda: ctx.gradient(n, q, qd, u, dqdd, qdd, minv, stream), stream)
        rows.append({"knots": n, "engine_us": round(t_eng, 2), "reference_kernel_us_dim3_32x7": round(t_ref, 2),
                     "reference_kernel_us_dim3_1x1": None if t_one is None else round(t_one, 2),
                     "engine_speedup_vs_32x7": round(t_ref / t_eng, 2)})
    print("\nREFERENCE_GPU_KERNEL_TIMING " + json.dumps(rows))
