"""CPU oracle of the learned field propagator (test infrastructure only).

The network has no counterpart in the reference; this file restates the
definition in include/phafd_fno.h in numpy (FP64 arithmetic) with a manual
backward pass.  With bf16=True it rounds to bfloat16 at the same points as
the GPU kernels (operands staged for the tensor cores, stored activations,
stored gradients), so GPU and oracle differ only by FP32 accumulation order
and transcendental implementations.  The manual backward is itself checked
against finite differences (tests/test_fno_oracle.py).

Parity status: no reference vectors exist for this component; the oracle is
pinned by finite differences and by the GPU agreeing with it."""
import numpy as np

C_CH, NKX, NK = 32, 8, 16
NMODE = NK * NK * NKX
LSZ = 1024 + 32 + NMODE * C_CH * C_CH * 2
SQ2PI = 0.7978845608028654


def bf16(a):
    """round to the nearest bfloat16 (ties to even), returned as float64"""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def ident(a):
    return np.asarray(a, np.float64)


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(SQ2PI * (x + 0.044715 * x ** 3)))


def gelu_d(x):
    t = np.tanh(SQ2PI * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * SQ2PI * (1.0 + 0.134145 * x * x)


def unpack(vec):
    v = np.asarray(vec, np.float64)
    p = {"P": v[0:512].reshape(32, 16), "pb": v[512:544]}
    base = 544
    for l in range(4):
        p["W%d" % l] = v[base:base + 1024].reshape(32, 32)
        p["b%d" % l] = v[base + 1024:base + 1056]
        p["R%d" % l] = v[base + 1056:base + LSZ].reshape(NMODE, 32, 32, 2)
        base += LSZ
    p["Q1"] = v[base:base + 1024].reshape(32, 32)
    p["q1b"] = v[base + 1024:base + 1056]
    p["q2"] = v[base + 1056:base + 1088]
    p["q2b"] = v[base + 1088]
    return p


def tables(nx, ny, nz, r):
    """x-stage tables (bfloat16 on the GPU) and y/z twiddles (FP32)."""
    x = np.arange(nx)
    F = np.zeros((16, nx))
    G = np.zeros((nx, 16))
    for kx in range(NKX):
        th = 2.0 * np.pi * ((kx * x) % nx) / nx
        c = np.cos(th).astype(np.float32).astype(np.float64)
        s = np.sin(th).astype(np.float32).astype(np.float64)
        w = 1.0 if kx == 0 else 2.0
        F[2 * kx] = r(c)
        F[2 * kx + 1] = r(-s)
        G[:, 2 * kx] = r((w * c).astype(np.float32))
        G[:, 2 * kx + 1] = r((-w * s).astype(np.float32))

    def tw(n):
        k = np.arange(NK)
        kk = np.where(k < NK // 2, k, k - NK)
        ph = (np.outer(kk, np.arange(n)) % n + n) % n
        th = 2.0 * np.pi * ph / n
        return np.cos(th).astype(np.float32) - 1j * np.sin(th).astype(np.float32)

    return F, G, tw(ny).astype(np.complex128), tw(nz).astype(np.complex128)


class FNOOracle:
    """phi, rho: arrays [nz][ny][nx]; norm as phafd_fno_set_norm."""

    def __init__(self, params, shape, norm, bf=True):
        self.p = unpack(params)
        self.nz, self.ny, self.nx = shape
        self.norm = np.asarray(norm, np.float64)
        self.r = bf16 if bf else ident
        self.F, self.G, self.ey, self.ez = tables(self.nx, self.ny, self.nz, self.r)
        self.N = self.nx * self.ny * self.nz
        self.Rc = [self.r(self.p["R%d" % l][..., 0]) + 1j * self.r(self.p["R%d" % l][..., 1]) for l in range(4)]

    def inputs(self, phi, rho, chi):
        n = self.norm.astype(np.float32)
        inp = np.zeros((self.nz, self.ny, self.nx, 16))
        inp[..., 0] = ((np.asarray(phi, np.float32) - n[0]) / n[1]).astype(np.float64)
        inp[..., 1] = ((np.asarray(rho, np.float32) - n[2]) / n[3]).astype(np.float64)
        inp[..., 2] = float(np.float32((np.float32(chi) - n[4]) / n[5]))
        return inp

    # truncated spectral convolution pieces
    def xdft(self, v, T):
        """x stage: [z,y,x,c] -> complex [z,y,kx,c] with table T [16][nx]"""
        re = np.einsum("kx,zyxc->zykc", T[0::2], v)
        im = np.einsum("kx,zyxc->zykc", T[1::2], v)
        return re + 1j * im

    def spectral_fwd(self, v, l):
        Vx = self.xdft(v, self.F)
        Vxy = np.einsum("zykc,qy->zqkc", Vx, self.ey)
        Vh = np.einsum("zqkc,pz->pqkc", Vxy, self.ez) / self.N
        R = self.Rc[l].reshape(NK, NK, NKX, 32, 32)
        Yh = np.einsum("pqkoi,pqki->pqko", R, Vh)
        Yxy = np.einsum("pqko,pz->zqko", Yh, np.conj(self.ez))
        Yx = np.einsum("zqko,qy->zyko", Yxy, np.conj(self.ey))
        Yr, Yi = self.r(Yx.real), self.r(Yx.imag)
        s = np.einsum("xk,zyko->zyxo", self.G[:, 0::2], Yr) + np.einsum("xk,zyko->zyxo", self.G[:, 1::2], Yi)
        return s, Vh

    def forward(self, phi, rho, chi):
        r, p = self.r, self.p
        cache = {}
        inp = r(self.inputs(phi, rho, chi))
        v = r(inp @ r(p["P"]).T + p["pb"])
        cache["inp"], cache["v"], cache["pre"], cache["vh"] = inp, [v], [], []
        for l in range(4):
            s, Vh = self.spectral_fwd(v, l)
            pre = v @ r(p["W%d" % l]).T + p["b%d" % l] + s
            cache["pre"].append(pre)
            cache["vh"].append(Vh)
            v = r(gelu(pre)) if l < 3 else r(pre)
            cache["v"].append(v)
        preh = v @ r(p["Q1"]).T + p["q1b"]
        out = gelu(preh) @ p["q2"] + p["q2b"]
        cache["preh"] = preh
        return out, cache

    def correction(self, phi, rho, chi):
        out, _ = self.forward(phi, rho, chi)
        return self.norm[6] * (out - out.mean())

    def loss_and_grad(self, phi, rho, chi, target):
        """loss = mean((out - target)^2) and the gradient dict (manual backward)"""
        r, p = self.r, self.p
        out, c = self.forward(phi, rho, chi)
        e = out - target
        loss = np.mean(e * e)
        gr = 2.0 * e / self.N
        g = {}
        preh = c["preh"]
        h = gelu(preh)
        g["q2"] = np.einsum("zyx,zyxk->k", gr, h)
        g["q2b"] = gr.sum()
        dph = gr[..., None] * p["q2"] * gelu_d(preh)
        g["q1b"] = dph.reshape(-1, 32).sum(0)
        dph = r(dph)
        v4 = c["v"][4]
        g["Q1"] = np.einsum("zyxk,zyxc->kc", dph, v4)
        delta = r(dph @ r(p["Q1"]))
        for l in range(3, -1, -1):
            vprev = c["v"][l]
            g["b%d" % l] = delta.reshape(-1, 32).sum(0)
            g["W%d" % l] = np.einsum("zyxo,zyxi->oi", delta, vprev)
            # adjoint of the spectral branch
            dYx = self.xdft(delta, self.G.T)           # x stage with G
            dYxy = np.einsum("zyko,qy->zqko", dYx, self.ey)
            dYh = np.einsum("zqko,pz->pqko", dYxy, self.ez)
            Vh = c["vh"][l]
            dR = dYh[..., :, None] * np.conj(Vh[..., None, :])   # [p,q,k,o,i]
            g["R%d" % l] = np.stack([dR.real, dR.imag], -1).reshape(NMODE, 32, 32, 2)
            R = self.Rc[l].reshape(NK, NK, NKX, 32, 32)
            dVh = np.einsum("pqkoi,pqko->pqki", np.conj(R), dYh)
            dVxy = np.einsum("pqki,pz->zqki", dVh, np.conj(self.ez)) / self.N
            dVx = np.einsum("zqki,qy->zyki", dVxy, np.conj(self.ey))
            dr, di = r(dVx.real), r(dVx.imag)
            gv = delta @ r(p["W%d" % l]) + np.einsum("kx,zyki->zyxi", self.F[0::2], dr) + \
                np.einsum("kx,zyki->zyxi", self.F[1::2], di)
            if l > 0:
                delta = r(gv * gelu_d(r(c["pre"][l - 1])))
            else:
                g["pb"] = gv.reshape(-1, 32).sum(0)
                g["P"] = np.einsum("zyxc,zyxj->cj", r(gv), c["inp"])
        return loss, g

    @staticmethod
    def flat(g):
        """gradient dict -> flat vector in the parameter layout"""
        v = np.zeros(544 + 4 * LSZ + 1089)
        v[0:512] = g["P"].reshape(-1)
        v[512:544] = g["pb"]
        base = 544
        for l in range(4):
            v[base:base + 1024] = g["W%d" % l].reshape(-1)
            v[base + 1024:base + 1056] = g["b%d" % l]
            v[base + 1056:base + LSZ] = g["R%d" % l].reshape(-1)
            base += LSZ
        v[base:base + 1024] = g["Q1"].reshape(-1)
        v[base + 1024:base + 1056] = g["q1b"]
        v[base + 1056:base + 1088] = g["q2"]
        v[base + 1088] = g["q2b"]
        return v
