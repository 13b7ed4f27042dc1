"""Either side of the gradient (GPU): external forces, forward dynamics only,
discrete-time Jacobians.  Checked against the FP64 oracle."""
import numpy as np
import pytest

import frg
import frg_oracle
from conftest import TOL, max_err

pytestmark = pytest.mark.gpu


def dev(torch, *arrs):
    return [torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda() for a in arrs]


@pytest.mark.parametrize("damping,mpc", [(0, 0), (1, 1)])
@pytest.mark.parametrize("n", [1, 33, 700])
def test_gradient_with_external_forces(damping, mpc, n):
    import torch
    q, qd, u = frg.sample_knots(n, seed=400 + n)
    rng = np.random.default_rng(n)
    fext = rng.uniform(-5, 5, (n, 42)).astype(np.float32)
    tq, tqd, tu, tf = dev(torch, q, qd, u, fext)
    out = [torch.empty((n, w), device="cuda") for w in (98, 7, 49)]
    with frg.Context(vel_damping=damping, mpc_mode=mpc) as ctx:
        ctx.gradient_fext(n, tq, tqd, tu, tf, *out)
        torch.cuda.synchronize()
    rd, rq, rm = frg_oracle.gradient_f64(q, qd, u, damping, mpc, fext=fext)
    assert max_err(out[0].cpu().numpy(), rd) <= TOL
    assert max_err(out[1].cpu().numpy(), rq) <= TOL
    assert max_err(out[2].cpu().numpy(), rm) <= TOL
    # the forces matter: without them q̈ differs
    _, rq0, _ = frg_oracle.gradient_f64(q, qd, u, damping, mpc)
    assert max_err(rq0, rq) > 1e-3


@pytest.mark.parametrize("with_fext", [False, True])
def test_forward_dynamics_only(with_fext):
    import torch
    n = 257
    q, qd, u = frg.sample_knots(n, seed=9)
    fext = np.random.default_rng(2).uniform(-3, 3, (n, 42)).astype(np.float32) if with_fext else None
    tq, tqd, tu = dev(torch, q, qd, u)
    tf = dev(torch, fext)[0] if with_fext else None
    qdd = torch.empty((n, 7), device="cuda")
    minv = torch.empty((n, 49), device="cuda")
    qdd2 = torch.empty((n, 7), device="cuda")
    with frg.Context() as ctx:
        ctx.forward_dynamics(n, tq, tqd, tu, qdd, minv, fext=tf)
        ctx.forward_dynamics(n, tq, tqd, tu, qdd2, None, fext=tf)  # Minv not wanted
        torch.cuda.synchronize()
    _, rq, rm = frg_oracle.gradient_f64(q, qd, u, fext=fext)
    assert max_err(qdd.cpu().numpy(), rq) <= TOL and max_err(minv.cpu().numpy(), rm) <= TOL
    assert torch.equal(qdd, qdd2)


def test_discrete_jacobians():
    import torch
    n, dt = 300, 0.01
    q, qd, u = frg.sample_knots(n, seed=77)
    tq, tqd, tu = dev(torch, q, qd, u)
    d, qq, m = (torch.empty((n, w), device="cuda") for w in (98, 7, 49))
    A = torch.empty((n, 196), device="cuda")
    B = torch.empty((n, 98), device="cuda")
    with frg.Context() as ctx:
        ctx.gradient(n, tq, tqd, tu, d, qq, m)
        ctx.discrete_jacobians(n, d, m, dt, A, B)
        torch.cuda.synchronize()
    rd, _, rm = frg_oracle.gradient_f64(q, qd, u)
    G = rd.reshape(n, 14, 7).transpose(0, 2, 1)  # [n, 7, 14]
    Aref = np.tile(np.eye(14), (n, 1, 1))
    Aref[:, :7, 7:] += dt * np.eye(7)
    Aref[:, 7:, :] += dt * G
    Bref = np.zeros((n, 14, 7))
    Bref[:, 7:, :] = dt * rm.reshape(n, 7, 7)
    Agot = A.cpu().numpy().reshape(n, 14, 14).transpose(0, 2, 1)
    Bgot = B.cpu().numpy().reshape(n, 7, 14).transpose(0, 2, 1)
    assert max_err(Agot.reshape(n, -1), Aref.reshape(n, -1)) <= TOL
    assert max_err(Bgot.reshape(n, -1), Bref.reshape(n, -1)) <= TOL


def test_discrete_jacobians_chunked_and_elementwise_agree():
    """16-byte-aligned arrays take the 64-knot chunk kernel (plus an
    element-wise tail); arrays one float off alignment take the element-wise
    kernel throughout.  Both give the same bits."""
    import torch
    n, dt = 1000, 0.02  # 15 chunks and a tail of 40 knots
    q, qd, u = frg.sample_knots(n, seed=78)
    tq, tqd, tu = dev(torch, q, qd, u)
    d, qq, m = (torch.empty((n, w), device="cuda") for w in (98, 7, 49))
    A = torch.empty((n, 196), device="cuda")
    B = torch.empty((n, 98), device="cuda")
    Abuf = torch.empty(n * 196 + 1, device="cuda")
    Bbuf = torch.empty(n * 98 + 1, device="cuda")
    A1, B1 = Abuf[1:].view(n, 196), Bbuf[1:].view(n, 98)
    with frg.Context() as ctx:
        ctx.gradient(n, tq, tqd, tu, d, qq, m)
        ctx.discrete_jacobians(n, d, m, dt, A, B)
        ctx.discrete_jacobians(n, d, m, dt, A1, B1)
        torch.cuda.synchronize()
    assert torch.equal(A, A1) and torch.equal(B, B1)


@pytest.mark.parametrize("damping,mpc", [(0, 0), (1, 1)])
@pytest.mark.parametrize("n", [1, 33, 1000])
def test_gradient_over_reference_knot_records(damping, mpc, n):
    """frg_gradient_knots on the reference's packed records [q|qd|u|qdd|Minv]
    (77 floats per knot): q̈ and Minv land in the records' fields and, with the
    gradient, carry the same bits as frg_gradient on separate arrays; q, qd, u
    are left as they were."""
    import torch
    q, qd, u = frg.sample_knots(n, seed=600 + n)
    rec = np.full((n, 77), np.nan, np.float32)
    rec[:, 0:7], rec[:, 7:14], rec[:, 14:21] = q, qd, u
    trec = torch.from_numpy(rec).cuda()
    tq, tqd, tu = dev(torch, q, qd, u)
    d_rec = torch.empty((n, 98), device="cuda")
    ref = [torch.empty((n, w), device="cuda") for w in (98, 7, 49)]
    with frg.Context(vel_damping=damping, mpc_mode=mpc) as ctx:
        ctx.gradient_knots(n, trec, d_rec)
        ctx.gradient(n, tq, tqd, tu, *ref)
        torch.cuda.synchronize()
    got = trec.cpu().numpy()
    assert np.array_equal(got[:, :21], rec[:, :21])
    assert np.array_equal(d_rec.cpu().numpy(), ref[0].cpu().numpy())
    assert np.array_equal(got[:, 21:28], ref[1].cpu().numpy())
    assert np.array_equal(got[:, 28:77], ref[2].cpu().numpy())
    rd, rq, rm = frg_oracle.gradient_f64(q, qd, u, damping, mpc)
    assert max_err(d_rec.cpu().numpy(), rd) <= TOL and max_err(got[:, 28:77], rm) <= TOL
