"""Differentiable torch restatement of the fused step -- TEST INFRASTRUCTURE ONLY.

The gradient oracle for the hand-written adjoint.  XLB differentiates its
stepper with Warp's tape (examples/out_of_core/subroutine/
autodiff_stepper_subroutine.py:460-466) or with jax.grad on the JAX backend;
neither Warp nor JAX is available here, so the reference gradient is torch
autograd through this restatement in float64, itself checked against central
finite differences and against the numpy oracle's forward step.

It restates oracle/lbm_oracle.step (same equations, same order of operations
where it matters for FP64 agreement) as a pure function of the population
field f and of the ZouHe / Regularized prescribed values:

    f_next = step(lat, f, aux, bc_mask, missing, omega, bcs, collision)

``aux`` is a float64 field of the grid's spatial shape; its value at a ZouHe /
Regularized cell is that cell's prescribed value (XLB keeps it in slot 0 of
f_1, boundary_condition.py:151-152, and carries it across steps by the aux
recovery of nse_stepper.py:318-342, so across steps it is a constant).  Cells
with id 255 are not supported (their populations are never written, so they
would make the step depend on the state two steps back).

Only ``tests/`` may import this module.
"""

import numpy as np
import torch

from oracle.lbm_oracle import Lattice, extrapolation_cs, normals_float  # noqa: F401

STREAMING = ("halfway_bb", "equilibrium", "zouhe_velocity", "zouhe_pressure", "regularized_velocity",
             "regularized_pressure", "extrapolation")


def pull(lat, f):
    """f_ps[l](x) = f[l](x - c_l), one-cell periodic wrap (stream.py:64-82)."""
    dims = tuple(range(lat.d))
    return torch.stack([torch.roll(f[l], tuple(int(v) for v in lat.c[:, l]), dims) for l in range(lat.q)])


def macroscopic(lat, f):
    rho = f[0]
    for l in range(1, lat.q):
        rho = rho + f[l]
    u = []
    for d in range(lat.d):
        acc = torch.zeros_like(rho)
        for l in range(lat.q):
            if lat.c[d, l] == 1:
                acc = acc + f[l]
            elif lat.c[d, l] == -1:
                acc = acc - f[l]
        u.append(acc / rho)
    return rho, u


def equilibrium(lat, rho, u):
    usq = u[0] * u[0]
    for d in range(1, lat.d):
        usq = usq + u[d] * u[d]
    usqr = 1.5 * usq
    out = []
    for l in range(lat.q):
        cu = torch.zeros_like(rho)
        for d in range(lat.d):
            if lat.c[d, l] == 1:
                cu = cu + u[d]
            elif lat.c[d, l] == -1:
                cu = cu - u[d]
        cu = cu * 3.0
        out.append(rho * float(lat.w[l]) * (1.0 + cu * (1.0 + 0.5 * cu) - usqr))
    return torch.stack(out)


def second_moment(lat, fneq):
    nt = lat.d * (lat.d + 1) // 2
    pi = []
    for t in range(nt):
        acc = torch.zeros_like(fneq[0])
        for q in range(lat.q):
            if lat.cc[q, t] == 1:
                acc = acc + fneq[q]
            elif lat.cc[q, t] == -1:
                acc = acc - fneq[q]
        pi.append(acc)
    return pi


def kbc(lat, f, feq, rho, omega):
    """kbc.py:192-296 (D2Q9 and D3Q27)."""
    fneq = f - feq
    pi = second_moment(lat, fneq)
    z = torch.zeros_like(rho)
    s = [z] * lat.q
    if lat.name == "D3Q27":
        nxz = pi[0] - pi[5]
        nyz = pi[3] - pi[5]
        a = (2.0 * nxz - nyz) / 6.0
        b = (-nxz + 2.0 * nyz) / 6.0
        cz = (-nxz - nyz) / 6.0
        for i, v in ((9, a), (18, a), (3, b), (6, b), (1, cz), (2, cz)):
            s[i] = v
        p1, p2, p4 = pi[1] / 4.0, pi[2] / 4.0, pi[4] / 4.0
        for i, v in ((12, p1), (24, p1), (21, -p1), (15, -p1), (10, p2), (20, p2), (19, -p2), (11, -p2),
                     (8, p4), (4, p4), (7, -p4), (5, -p4)):
            s[i] = v
        delta_s = torch.stack(s) * rho
    elif lat.name == "D2Q9":
        n = pi[0] - pi[2]
        for i, v in ((3, n), (6, n), (2, -n), (1, -n), (8, pi[1]), (4, -pi[1]), (5, -pi[1]), (7, pi[1])):
            s[i] = v
        delta_s = torch.stack(s) * rho / 4.0
    else:
        raise NotImplementedError(lat.name)
    beta = 0.5 * omega
    inv_beta = 1.0 / beta
    delta_h = fneq - delta_s
    temp = delta_h / feq
    sp1 = (temp * delta_s).sum(0)
    sp2 = (temp * delta_h).sum(0)
    gamma = inv_beta - (2.0 - inv_beta) * sp1 / (1e-32 + sp2)
    return f - beta * (2.0 * delta_s + gamma * delta_h)


def _bc_fsum(lat, f, miss):
    known = torch.zeros_like(f[0])
    middle = torch.zeros_like(f[0])
    for l in range(lat.q):
        k = torch.as_tensor(miss[lat.opp[l]])
        m = torch.as_tensor((~miss[lat.opp[l]]) & (~miss[l]))
        known = torch.where(k, known + 2.0 * f[l], known)
        middle = torch.where(m, middle + f[l], middle)
    return known + middle


def zouhe_like(lat, f, miss, aux, kind):
    """bc_zouhe.py:279-343, bc_regularized.py:134-202; f (Q, n), miss (Q, n) numpy bool, aux (n,)."""
    nv = normals_float(lat, miss, np.float64).astype(np.float64)
    nvt = [torch.as_tensor(nv[d], dtype=f.dtype, device=f.device) for d in range(lat.d)]
    fsum = _bc_fsum(lat, f, miss)
    if kind.endswith("velocity"):
        u = [(-aux) * nvt[d] for d in range(lat.d)]
        unormal = torch.zeros_like(fsum)
        for d in range(lat.d):
            unormal = unormal + u[d] * nvt[d]
        rho = fsum / (1.0 + unormal)
    else:
        rho = aux
        unormal = -1.0 + fsum / rho
        u = [unormal * nvt[d] for d in range(lat.d)]
    feq = equilibrium(lat, rho, u)
    g = list(f)
    for l in range(lat.q):  # in place and in order, as XLB's loop (helper_functions_bc.py:263-272)
        o = lat.opp[l]
        g[l] = torch.where(torch.as_tensor(miss[l]), g[o] + feq[l] - feq[o], g[l])
    out = torch.stack(g)
    if kind.startswith("regularized"):
        pi = second_moment(lat, out - feq)
        rows = []
        for l in range(lat.q):
            acc = torch.zeros_like(fsum)
            for t in range(len(pi)):
                if lat.qi[l, t] != 0.0:
                    acc = acc + float(lat.qi[l, t]) * pi[t]
            rows.append(feq[l] + 4.5 * float(lat.w[l]) * acc)
        out = torch.stack(rows)
    return out


def step(lat, f, aux, bc_mask, missing, omega, bcs, collision="BGK"):
    """One step of the fused stepper as a differentiable function of (f, aux).

    f: float64 (Q, *shape); aux: float64 (*shape); bc_mask (1, *shape) and
    missing (Q, *shape) numpy arrays; bcs: oracle.lbm_oracle.BC list."""
    if (bc_mask == 255).any():
        raise NotImplementedError("cells with id 255 are not differentiated")
    q = lat.q
    shp = tuple(f.shape[1:])
    ids = bc_mask[0].reshape(-1)
    miss_all = missing.reshape(q, -1)
    own = f.reshape(q, -1)
    flat = pull(lat, f).reshape(q, -1)
    auxf = aux.reshape(-1)
    dev = f.device
    for bc in bcs:
        if bc.kind not in STREAMING:
            continue
        sel = np.nonzero(ids == bc.id)[0]
        if len(sel) == 0:
            continue
        st = torch.as_tensor(sel, device=dev)
        fp = flat[:, st]
        miss = miss_all[:, sel]
        if bc.kind in ("halfway_bb", "extrapolation"):
            own_s = own[:, st]
            fp = torch.stack([torch.where(torch.as_tensor(miss[l], device=dev), own_s[lat.opp[l]], fp[l]) for l in range(q)])
        elif bc.kind == "equilibrium":
            rho = torch.full((len(sel),), float(bc.rho), dtype=f.dtype, device=dev)
            u = [torch.full((len(sel),), float(bc.u[d]), dtype=f.dtype, device=dev) for d in range(lat.d)]
            fp = equilibrium(lat, rho, u)
        else:
            fp = zouhe_like(lat, fp, miss, auxf[st], bc.kind)
        flat = flat.index_copy(1, st, fp)

    rho, u = macroscopic(lat, flat)
    feq = equilibrium(lat, rho, u)
    if collision in ("BGK", "BGK_PAIR"):
        fout = flat - omega * (flat - feq)
    elif collision == "KBC":
        fout = kbc(lat, flat, feq, rho, omega)
    else:
        raise ValueError(collision)

    for bc in bcs:
        sel = np.nonzero(ids == bc.id)[0]
        if len(sel) == 0:
            continue
        st = torch.as_tensor(sel, device=dev)
        if bc.kind == "fullway_bb":
            fout = fout.index_copy(1, st, flat[:, st][list(lat.opp)])
        elif bc.kind == "extrapolation":
            cs = float(extrapolation_cs(np.float64))
            miss = miss_all[:, sel]
            cells = np.array(np.unravel_index(sel, shp))
            nv = normals_float(lat, miss, np.float64)
            rows = list(fout[:, st])
            fp = flat[:, st]
            for l in range(q):
                if not miss[l].any():
                    continue
                src = cells.copy()
                for d in range(lat.d):
                    src[d] = (src[d] - (lat.c[d, l] + nv[d])) % shp[d]
                lin = torch.as_tensor(np.ravel_multi_index(tuple(src), shp), device=dev)
                f_aux = own[l][lin]
                o = lat.opp[l]
                rows[o] = torch.where(torch.as_tensor(miss[l], device=dev), (1.0 - cs) * fp[l] + cs * f_aux, rows[o])
            fout = fout.index_copy(1, st, torch.stack(rows))
    return fout.reshape((q,) + shp)


def run(lat, f, aux, bc_mask, missing, omega, bcs, steps, collision="BGK"):
    for _ in range(steps):
        f = step(lat, f, aux, bc_mask, missing, omega, bcs, collision)
    return f


def aux_field(lat, shape3, bc_mask, f1_decoded_slot0, bcs):
    """The aux field the step reads: slot 0 of the initial f_1 at ZouHe /
    Regularized cells, zero elsewhere (float64 numpy, spatial shape)."""
    out = np.zeros(shape3, dtype=np.float64)
    for bc in bcs:
        if bc.kind.startswith("zouhe") or bc.kind.startswith("regularized"):
            m = bc_mask[0] == bc.id
            out[m] = f1_decoded_slot0[m]
    return out
