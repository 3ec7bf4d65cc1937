"""Test infrastructure: the frozen-mesh Kelvin-Helmholtz step of the library
restated in PyTorch FP64 on the global periodic 256^2 grid, so that
torch.autograd gives an independent reference gradient for the discrete
adjoint.  On a uniform periodic mesh the block decomposition is invisible:
ghost cells are copies of the neighbours' interiors, so MUSCL2D.cpp:24-116
(with celledges.cpp:38-43 and the MC limiter, slopelimiter.cpp:23-27), the
Rusanov flux (riemannS.cpp:58-116), the residual and RK2 (main.cpp:147-189),
and CT2D.cpp:16-120 become periodic stencils.  Arrays are indexed [.., ix, iy];
face arrays hold the face at the left (x) / bottom (y) of cell (ix, iy).
"""
import math

import numpy as np
import torch

EPS = 1.0e-15


class BranchTape:
    """Branches of the piecewise-smooth parts of the step: the MC limiter
    (which of 0, 2r, (1+r)/2, 2 it returns), the larger of the two Rusanov
    wave speeds and the sign inside |u|.  mode "record" appends the branch of
    every evaluation; mode "replay" evaluates each with the recorded branch
    instead of its own, i.e. the smooth map of the recorded run, whose
    central differences converge to the derivative the adjoint computes;
    `flips` counts evaluations whose own branch differs from the recorded
    one.  mode None: the plain step."""

    def __init__(self):
        self.mode, self.rec, self.pos, self.flips, self.evals = None, [], 0, 0, 0

    def start(self, mode):
        self.mode, self.pos, self.flips, self.evals = mode, 0, 0, 0
        if mode == "record":
            self.rec = []

    def branch(self, own):
        """own: the branch index tensor of this evaluation; returns the one to use"""
        if self.mode is None:
            return own
        if self.mode == "record":
            self.rec.append(own.to(torch.int8))
            return own
        r = self.rec[self.pos].to(own.dtype)
        self.pos += 1
        self.flips += int((r != own).sum())
        self.evals += own.numel()
        return r


TAPE = BranchTape()


def kh_ic(a, n=256, gamma=5.0 / 3.0):
    """U [8, n, n], Bx, By [n, n] of the KH layer with perturbation amplitudes
    a (16) on [0,1]^2 (cell centres (i + 1/2) / n)."""
    dt = a.dtype
    x = (torch.arange(n, dtype=dt, device=a.device) + 0.5) / n
    X, Y = torch.meshgrid(x, x, indexing="ij")
    inside = (Y - 0.5).abs() <= 0.25
    rho = torch.where(inside, torch.full_like(X, 2.0), torch.full_like(X, 1.0))
    u = torch.where(inside, torch.full_like(X, 0.5), torch.full_like(X, -0.5))
    env = torch.exp(-(Y - 0.25) ** 2 / 0.01) + torch.exp(-(Y - 0.75) ** 2 / 0.01)
    k = torch.arange(1, 17, dtype=dt, device=a.device)
    v = (a[:, None, None] * torch.sin(2.0 * math.pi * k[:, None, None] * X[None])).sum(0) * env
    p = torch.full_like(X, 2.5)
    bx = torch.full_like(X, 0.1 / math.sqrt(4.0 * math.pi))
    zero = torch.zeros_like(X)
    E = p / (gamma - 1) + 0.5 * rho * (u * u + v * v) + 0.5 * bx * bx
    U = torch.stack([rho, rho * u, rho * v, zero, E, bx, zero, zero])
    return U, bx.clone(), zero.clone()


def prim(U, g):
    rho = U[0]
    v = U[1:4] / rho
    p = (g - 1) * (U[4] - 0.5 * rho * (v * v).sum(0)) - (g - 1) * 0.5 * (U[5:8] * U[5:8]).sum(0)
    return torch.cat([rho[None], v, p[None], U[5:8]])


def mc(r):
    """slopelimiter.cpp:23-27, max(0, min(2r, (1+r)/2, 2))"""
    a, b = 2.0 * r, 0.5 * (1.0 + r)
    v = torch.clamp(torch.minimum(torch.minimum(a, b), torch.full_like(r, 2.0)), min=0.0)
    if TAPE.mode is None:
        return v
    own = torch.where(v == 0.0, 0, torch.where(v == a, 1, torch.where(v == b, 2, 3)))
    br = TAPE.branch(own)
    return torch.where(br == 0, torch.zeros_like(r), torch.where(br == 1, a, torch.where(br == 2, b, torch.full_like(r, 2.0))))


def tabs(x):
    """|x| with its sign branch on the tape"""
    if TAPE.mode is None:
        return x.abs()
    br = TAPE.branch((x < 0).to(torch.int64))
    return torch.where(br == 1, -x, x)


def tmax(a, b):
    """max(a, b) with its branch on the tape"""
    if TAPE.mode is None:
        return torch.maximum(a, b)
    br = TAPE.branch((b > a).to(torch.int64))
    return torch.where(br == 1, b, a)


def faces(W, d):
    """MUSCL states at the face m+1/2 along dim d (1 = x, 2 = y of W [8, n, n])."""
    Wm = torch.roll(W, 1, d)
    Wp = torch.roll(W, -1, d)
    Wpp = torch.roll(W, -2, d)
    dA, dB, dC = W - Wm, Wp - W, Wpp - Wp
    left = W + 0.5 * mc(dB / (dA + EPS)) * dA
    right = Wp - 0.5 * mc(dB / (dC + EPS)) * dC
    return left, right


def rusanov_x(wl, wr, g):
    def side(w):
        rho, u, v, z, p, bx, by, bz = w
        b2 = bx * bx + by * by + bz * bz
        C, A, T = b2 / rho, g * p / rho, (by * by + bz * bz) / rho
        cf = torch.sqrt(0.5 * (C + A + torch.sqrt((C - A) ** 2 + 4.0 * A * T)))
        e = p / (g - 1) + 0.5 * rho * (u * u + v * v + z * z) + 0.5 * b2
        pt = p + 0.5 * b2
        q = torch.stack([rho, rho * u, rho * v, rho * z, e, bx, by, bz])
        F = torch.stack([rho * u, rho * u * u + pt - bx * bx, rho * u * v - bx * by, rho * u * z - bx * bz,
                         u * (e + pt) - bx * (u * bx + v * by + z * bz), torch.zeros_like(rho),
                         u * by - bx * v, u * bz - bx * z])
        return q, F, cf
    qL, FL, cL = side(wl)
    qR, FR, cR = side(wr)
    im = tmax(cL + tabs(wl[1]), cR + tabs(wr[1]))
    return 0.5 * (FL + FR) - 0.5 * im * (qR - qL)


SWAP = [0, 2, 1, 3, 4, 6, 5, 7]


def fluxes(U, Bx, By, g):
    """x fluxes at faces m+1/2 (Fr[:, m, j]) and y fluxes (Gr[:, i, m])."""
    W = prim(U, g)
    l, r = faces(W, 1)
    bn = torch.roll(Bx, -1, 0)
    l = torch.cat([l[:5], bn[None], l[6:]])
    r = torch.cat([r[:5], bn[None], r[6:]])
    Fr = rusanov_x(l, r, g)
    l, r = faces(W, 2)
    bn = torch.roll(By, -1, 1)
    l = torch.cat([l[:6], bn[None], l[7:]])[SWAP]
    r = torch.cat([r[:6], bn[None], r[7:]])[SWAP]
    Gr = rusanov_x(l, r, g)[SWAP]
    return Fr, Gr


def emf(Fr, Gr):
    """E at the corner (i-1/2, j-1/2) (CT2D.cpp:19-22)."""
    G5, F6 = Gr[5], Fr[6]
    return 0.25 * ((torch.roll(G5, (1, 1), (0, 1)) + torch.roll(G5, 1, 1)) -
                   (torch.roll(F6, (1, 1), (0, 1)) + torch.roll(F6, 1, 0)))


def curl(E, dx, dy):
    return (torch.roll(E, -1, 1) - E) / dy, -(torch.roll(E, -1, 0) - E) / dx


def correct(U, Bx, By):
    bx = 0.5 * (Bx + torch.roll(Bx, -1, 0))
    by = 0.5 * (By + torch.roll(By, -1, 1))
    E = U[4] + 0.5 * ((bx * bx + by * by) - (U[5] * U[5] + U[6] * U[6]))
    return torch.stack([U[0], U[1], U[2], U[3], E, bx, by, U[7]])


def step(U, Bx, By, dt, g, dx):
    Fr, Gr = fluxes(U, Bx, By, g)
    res = (Fr - torch.roll(Fr, 1, 1)) / dx + (Gr - torch.roll(Gr, 1, 2)) / dx
    Us = U - dt * res
    cx, cy = curl(emf(Fr, Gr), dx, dx)
    Bxs, Bys = Bx - dt * cx, By - dt * cy
    Us = correct(Us, Bxs, Bys)
    Fr, Gr = fluxes(Us, Bxs, Bys, g)
    res = (Fr - torch.roll(Fr, 1, 1)) / dx + (Gr - torch.roll(Gr, 1, 2)) / dx
    Un = 0.5 * (U + Us - dt * res)
    cx, cy = curl(emf(Fr, Gr), dx, dx)
    Bxn, Byn = 0.5 * (Bx + Bxs - dt * cx), 0.5 * (By + Bys - dt * cy)
    return correct(Un, Bxn, Byn), Bxn, Byn


def box_mask(n=256, lo=0.4, hi=0.6, dtype=torch.float64, device="cpu"):
    """dA on the cells whose centre lies in [lo, hi]^2, else 0."""
    x = (torch.arange(n, dtype=dtype, device=device) + 0.5) / n
    m = ((x >= lo) & (x <= hi)).to(dtype)
    return m[:, None] * m[None, :] / (n * n)


def to_blocks(A, icoord, ng=2, nb=16):
    """Global [nv, n, n] array -> [blocks][nv][nb+2ng][nb+2ng] ([j][i] planes)
    with periodic ghost cells, block origins from icoord (cells)."""
    A = np.asarray(A)
    nv, n, _ = A.shape
    N = nb + 2 * ng
    out = np.empty((len(icoord), nv, N, N))
    idx = np.arange(N) - ng
    for b, (x0, y0) in enumerate(icoord):
        ii = (x0 + idx) % n
        jj = (y0 + idx) % n
        out[b] = A[:, ii][:, :, jj].transpose(0, 2, 1)
    return out


def from_blocks(Ab, icoord, n=256, ng=2, nb=16):
    """Interior cells of [blocks][nv][N][N] -> global [nv, n, n]."""
    nv = Ab.shape[1]
    out = np.zeros((nv, n, n))
    for b, (x0, y0) in enumerate(icoord):
        out[:, x0:x0 + nb, y0:y0 + nb] = Ab[b, :, ng:ng + nb, ng:ng + nb].transpose(0, 2, 1)
    return out
