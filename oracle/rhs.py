"""FP64 RHS operators in the reference's own unfused form (oracle; test
infrastructure).

Each function takes the oracle discretisation and per-field ``(Nel, Np)``
arrays and returns the RHS fields in the same layout.  On triangle meshes
(``d.dim == 2``) the same code runs with two-component vectors; Maxwell then
takes the TM fields (E_z, H_x, H_y), grudge's field subset for
``dimensions=2``.
"""

from __future__ import annotations

import numpy as np

from oracle.geometry import OracleDisc


# {{{ grudge primitives (affine elements, nodal base discretisation)


def weak_grad(d: OracleDisc, u: np.ndarray) -> np.ndarray:
    """``op.weak_local_grad``: out[x, e, i] = sum_r ST_r (J dr/dx_x u)."""
    return np.einsum("rij,erx,ej->xei", d.ops.stiff_t, d.jg, u)


def weak_div(d: OracleDisc, v: np.ndarray) -> np.ndarray:
    """``op.weak_local_div`` over the leading (x) axis of ``v``."""
    return np.einsum("rij,erx,xej->ei", d.ops.stiff_t, d.jg, v)


def local_grad(d: OracleDisc, u: np.ndarray) -> np.ndarray:
    """Strong ``op.local_d_dx`` for every x: sum_r dr/dx_x D_r u."""
    return np.einsum("erx,rij,ej->xei", d.metric, d.ops.diff, u)


def face_mass(d: OracleDisc, flux: np.ndarray) -> np.ndarray:
    """``op.face_mass`` of an all-faces field ``flux`` (Nel, F, Nfp)."""
    return np.einsum("kfj,ef,efj->ek", d.ops.face_mass, d.sj, flux)


def inverse_mass(d: OracleDisc, x: np.ndarray) -> np.ndarray:
    """``op.inverse_mass``: (1/J) M^-1 x."""
    minv = np.linalg.inv(d.ops.mass)
    return np.einsum("ij,ej->ei", minv, x) / d.jac[:, None]


def traces(d: OracleDisc, u: np.ndarray):
    flat = u.reshape(-1)
    return flat[d.int_idx], flat[d.ext_idx]


# }}}


def wave_rhs(d: OracleDisc, u: np.ndarray, v: np.ndarray, c: float = 1.0,
             parts: bool = False):
    """``actx_dgfem_suite/equations/wave.py:121-200`` with ``quad_tag=None``.

    Returns ``(rhs_u (Nel, Np), rhs_v (dim, Nel, Np))``; with ``parts=True``
    returns ``(rhs (1 + dim, Nel, Np), volume part, surface part)`` where the
    parts are the inverse-mass images of the volume and face-mass terms."""
    dim = d.dim
    n = d.normal.transpose(2, 0, 1)[..., None]            # (dim, Nel, F, 1)
    ui, ue = traces(d, u)
    vi = np.empty((dim,) + ui.shape)
    ve = np.empty_like(vi)
    for x in range(dim):
        vi[x], ve[x] = traces(d, v[x])
    # boundary pair (wave.py:152-156, 177-182): interior (u, v), exterior (-u, v)
    b = d.bdry[..., None]
    ue = np.where(b, -ui, ue)
    ve = np.where(b[None], vi, ve)

    # wave_flux (wave.py:80-114)
    v_avg = 0.5 * (vi + ve)
    u_avg = 0.5 * (ui + ue)
    u_diff = ue - ui
    v_diff = ve - vi
    flux_u = (v_avg * n).sum(axis=0)
    flux_v = u_avg[None] * n
    v_jump = (v_diff * n).sum(axis=0)
    flux_u = flux_u + 0.5 * u_diff
    flux_v = flux_v + 0.5 * v_jump[None] * n
    flux_u = c * flux_u
    flux_v = c * flux_v

    rhs_u = inverse_mass(d, -c * weak_div(d, v) + face_mass(d, flux_u))
    wg = weak_grad(d, u)
    rhs_v = np.stack([inverse_mass(d, -c * wg[x] + face_mass(d, flux_v[x]))
                      for x in range(dim)])
    if parts:
        vol = np.stack([inverse_mass(d, -c * weak_div(d, v))]
                       + [inverse_mass(d, -c * wg[x]) for x in range(dim)])
        surf = np.stack([inverse_mass(d, face_mass(d, flux_u))]
                        + [inverse_mass(d, face_mass(d, flux_v[x])) for x in range(dim)])
        return np.concatenate([rhs_u[None], rhs_v]), vol, surf
    return rhs_u, rhs_v


# {{{ Euler


def _pressure(rho, rho_e, rho_u, gamma):
    return (gamma - 1.0) * (rho_e - 0.5 * (rho_u * rho_u).sum(axis=0) / rho)


def _volume_flux(rho, rho_e, rho_u, gamma):
    """grudge ``euler_volume_flux``: per conserved field, a dim-vector over x.
    Returns (2 + dim, dim, ...) ordered mass, energy, momentum_0..dim-1."""
    p = _pressure(rho, rho_e, rho_u, gamma)
    u = rho_u / rho
    out = [rho_u, u * (rho_e + p)]
    for i in range(rho_u.shape[0]):
        row = rho_u[i][None] * u
        row = row.copy()
        row[i] = row[i] + p
        out.append(row)
    return np.stack(out)


def _wavespeed(rho, rho_e, rho_u, gamma):
    p = _pressure(rho, rho_e, rho_u, gamma)
    u = rho_u / rho
    return np.sqrt((u * u).sum(axis=0)) + np.sqrt(gamma * (p / rho))


def euler_rhs(d: OracleDisc, q: np.ndarray, gamma: float = 1.4,
              parts: bool = False):
    """grudge ``EulerOperator.operator`` (flux_type "lf", InviscidWallBC on
    all boundaries, no over-integration), as set up at
    ``actx_dgfem_suite/equations/euler.py:168-179``.

    ``q``: (2 + dim, Nel, Np) ordered mass, energy, momentum_x, momentum_y
    (, momentum_z).  Returns the RHS in the same layout (with ``parts=True``:
    ``(rhs, volume part, surface part)``)."""
    dim = d.dim
    nf = 2 + dim
    rho, rho_e, rho_u = q[0], q[1], q[2:nf]
    fvol = _volume_flux(rho, rho_e, rho_u, gamma)          # (nf, dim, Nel, Np)
    volume = np.stack([weak_div(d, fvol[k]) for k in range(nf)])

    qi = np.empty((nf,) + d.int_idx.shape)
    qe = np.empty_like(qi)
    for k in range(nf):
        qi[k], qe[k] = traces(d, q[k])
    n = d.normal.transpose(2, 0, 1)                        # (dim, Nel, F)
    # InviscidWallBC: mirror the normal momentum
    mom_i = qi[2:nf]
    mn = (mom_i * n[..., None]).sum(axis=0)
    mom_wall = mom_i - 2.0 * n[..., None] * mn[None]
    b = d.bdry[..., None]
    qe[0] = np.where(b, qi[0], qe[0])
    qe[1] = np.where(b, qi[1], qe[1])
    qe[2:nf] = np.where(b[None], mom_wall, qe[2:nf])

    fi = _volume_flux(qi[0], qi[1], qi[2:nf], gamma)       # (nf, dim, Nel, F, Nfp)
    fe = _volume_flux(qe[0], qe[1], qe[2:nf], gamma)
    lam = np.maximum(_wavespeed(qi[0], qi[1], qi[2:nf], gamma),
                     _wavespeed(qe[0], qe[1], qe[2:nf], gamma))
    num = 0.5 * (fi + fe)                                  # flux_tpair.avg
    num = num - lam[None, None] * (qe - qi)[:, None] * n[None, :, :, :, None] / 2
    fn = (num * n[None, :, :, :, None]).sum(axis=1)        # num_flux @ normal

    rhs = np.stack([inverse_mass(d, volume[k] - face_mass(d, fn[k]))
                    for k in range(nf)])
    if parts:
        vol = np.stack([inverse_mass(d, volume[k]) for k in range(nf)])
        surf = np.stack([inverse_mass(d, -face_mass(d, fn[k])) for k in range(nf)])
        return rhs, vol, surf
    return rhs


# }}}


# {{{ Maxwell


def _cross(a, b):
    return np.stack([a[1] * b[2] - a[2] * b[1],
                     a[2] * b[0] - a[0] * b[2],
                     a[0] * b[1] - a[1] * b[0]])


def maxwell_rhs(d: OracleDisc, w: np.ndarray, alpha: float = 0.5,
                epsilon: float = 1.0, mu: float = 1.0, parts: bool = False):
    """grudge ``MaxwellOperator.operator`` (3D, constant material, numeric
    flux_type ``alpha``, PEC on all boundaries), as set up at
    ``actx_dgfem_suite/equations/maxwell.py:55-70``.

    ``w``: (6, Nel, Np) ordered E_x, E_y, E_z, H_x, H_y, H_z; on triangle
    meshes (3, Nel, Np) ordered E_z, H_x, H_y (TM fields), evaluated as the
    3D operator on E = (0, 0, E_z), H = (H_x, H_y, 0) with no z-dependence."""
    if d.dim == 2:
        return _maxwell_tm(d, w, alpha, epsilon, mu, parts)
    e, h = w[:3], w[3:]
    de = np.stack([local_grad(d, e[k]) for k in range(3)])  # [k, x]
    dh = np.stack([local_grad(d, h[k]) for k in range(3)])
    curl_e = np.stack([de[2, 1] - de[1, 2], de[0, 2] - de[2, 0], de[1, 0] - de[0, 1]])
    curl_h = np.stack([dh[2, 1] - dh[1, 2], dh[0, 2] - dh[2, 0], dh[1, 0] - dh[0, 1]])

    wi = np.empty((6,) + d.int_idx.shape)
    we = np.empty_like(wi)
    for k in range(6):
        wi[k], we[k] = traces(d, w[k])
    b = d.bdry[None, ..., None]
    # pec_bc: exterior (-E, H)
    we[:3] = np.where(b, -wi[:3], we[:3])
    we[3:] = np.where(b, wi[3:], we[3:])
    n = d.normal.transpose(2, 0, 1)[..., None]             # (3, Nel, 4, 1)
    z = np.sqrt(mu / epsilon)
    y = 1.0 / z
    je = we[:3] - wi[:3]
    jh = we[3:] - wi[3:]
    flux_e = -1.0 / (z + z) * _cross(n, z * jh - alpha * _cross(n, je))
    flux_h = 1.0 / (y + y) * _cross(n, y * je + alpha * _cross(n, jh))
    fl = np.concatenate([flux_e, flux_h])
    lifted = np.stack([inverse_mass(d, face_mass(d, fl[k])) for k in range(6)])
    local = np.concatenate([-curl_h, curl_e])
    div = np.array([epsilon] * 3 + [mu] * 3)[:, None, None]
    rhs = (-local - lifted) / div
    if parts:
        return rhs, -local / div, -lifted / div
    return rhs


# }}}


def _maxwell_tm(d: OracleDisc, w: np.ndarray, alpha: float, epsilon: float,
                mu: float, parts: bool):
    """2D TM restriction of :func:`maxwell_rhs`: curl H = (0, 0, dHy/dx -
    dHx/dy), curl E = (dEz/dy, -dEz/dx, 0), the same alpha flux on 3-vectors
    with n_z = 0 and the PEC mirror; returns (E_z, H_x, H_y)."""
    ez, hx, hy = w
    dez, dhx, dhy = (local_grad(d, f) for f in (ez, hx, hy))   # [x] each
    curl_h_z = dhy[0] - dhx[1]
    curl_e = (dez[1], -dez[0])
    wi = np.empty((3,) + d.int_idx.shape)
    we = np.empty_like(wi)
    for k in range(3):
        wi[k], we[k] = traces(d, w[k])
    b = d.bdry[..., None]
    we[0] = np.where(b, -wi[0], we[0])                      # E_ext = -E
    we[1:] = np.where(b[None], wi[1:], we[1:])              # H_ext = H
    nx, ny = (d.normal[:, :, x][..., None] for x in range(2))
    zero = np.zeros_like(nx * wi[0])
    n = np.stack([nx + zero, ny + zero, zero])
    z = np.sqrt(mu / epsilon)
    y = 1.0 / z
    je = np.stack([zero, zero, we[0] - wi[0]])
    jh = np.stack([we[1] - wi[1], we[2] - wi[2], zero])
    flux_e = -1.0 / (z + z) * _cross(n, z * jh - alpha * _cross(n, je))
    flux_h = 1.0 / (y + y) * _cross(n, y * je + alpha * _cross(n, jh))
    fl = [flux_e[2], flux_h[0], flux_h[1]]
    lifted = np.stack([inverse_mass(d, face_mass(d, f)) for f in fl])
    local = np.stack([-curl_h_z, curl_e[0], curl_e[1]])
    div = np.array([epsilon, mu, mu])[:, None, None]
    rhs = (-local - lifted) / div
    if parts:
        return rhs, -local / div, -lifted / div
    return rhs
