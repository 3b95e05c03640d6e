"""CPU FP64 restatement of lprec's log-polar Radon transform (the oracle).

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this
module, and only as the checker or as the timed CPU baseline.  The product
(``lprec_gb300``) never imports it; its GPU path fails loudly when the CUDA
library is missing.

What it restates (all paths relative to the lprec project):

* geometry      -- src/lprec/initsgl.py:25-99   (create_gl, getparameters, osg, splineB3)
* fwd tables    -- src/lprec/initsfwd.py:15-93  (create_fwd, fzeta_loop_weights)
* adj tables    -- src/lprec/initsadj.py:19-203 (create_adj, fzeta_loop_weights_adj,
                                                 take_filter, wint)
* prefilter     -- src/include/main_kernels.cuh:97-185, src/cuda/lpRgpu.cu:219-240
* interpolation -- src/include/main_kernels.cuh:9-84 (wrap addressing, texel centre
                   shift, cubic B-spline built from bilinear fetches)
* pipelines     -- src/cuda/lpRgpu.cu:243-330 (execFwd / execAdj)
* wrappers      -- src/cuda/lpRgpu.cu:163-216 (cor window, osangles step, padker)
* FBP filter    -- src/cuda/lpRgpu.cu:333-382, src/include/simple_kernels.cuh:37-85
* solvers       -- src/lprec/lpmethods.py:7-338

Arithmetic: every table is computed in float64 from the reference formulas and
may be rounded once to float32 (``round_tables``); the transforms themselves
run in float64 with exact interpolation weights.  The reference's texture unit
quantises bilinear fractions to 8 bits; this restatement does not (an optional
``tex8`` flag reproduces that quantisation for comparison only).

Pinned against the reference's own tests (tests/test_adj_many.py and
tests/test_adj_ptr.py tolerances) and against the reference's own precompute,
imported with NumPy standing in for CuPy (tests/golden/make_golden.py).
"""
import math
import numpy as np

NSPAN = 3
POLE = math.sqrt(3.0) - 2.0          # main_kernels.cuh:2
LAMBDA = (1.0 - POLE) * (1.0 - 1.0 / POLE)


# --------------------------------------------------------------------------
# geometry (initsgl.py)
# --------------------------------------------------------------------------
class Geometry:
    pass


def osg(aR, theta):
    """initsgl.py:73-77."""
    t = np.linspace(-np.pi / 2, np.pi / 2, 1000)
    w = aR * np.cos(t) + (1 - aR) + 1j * aR * np.sin(t)
    return max(np.log(abs(w)) + np.log(np.cos(theta - np.arctan2(w.imag, w.real))))


def splineB3(x2, r):
    """initsgl.py:80-99 (cubic B-spline samples centred on the grid)."""
    x2 = np.asarray(x2)
    sizex = len(x2)
    x2 = x2 - (x2[-1] + x2[0]) / 2
    stepx = x2[1] - x2[0]
    ri = int(np.ceil(2 * r))
    r = r * stepx
    c = int(np.ceil((sizex + 1) / 2.0)) - 1
    x2c = x2[c]
    x = x2[c - ri:c + ri + 1]
    d = np.abs(x - x2c) / r
    B3 = x * 0
    for ix in range(-ri, ri + 1):
        i = ix + ri
        if d[i] < 1:
            B3[i] = (3 * d[i] ** 3 - 6 * d[i] ** 2 + 4) / 6
        elif d[i] < 2:
            B3[i] = (-d[i] ** 3 + 6 * d[i] ** 2 - 12 * d[i] + 8) / 6
    B3f = x2 * 0
    B3f[c - ri:c + ri + 1] = B3
    return B3f


def create_geometry(N0, Nproj, Nslices, cor, interp_type):
    """initsgl.py:25-70.  thsp/rhosp/erho are float32 as in the reference."""
    G = Geometry()
    G.Nspan = NSPAN
    G.beta = np.pi / NSPAN
    G.N0 = int(N0)
    G.N = int(np.ceil((N0 + abs(N0 / 2 - cor) * 2.0) / 16.0) * 16)
    G.osangles = int(max(round(3.0 * G.N / 2.0 / Nproj), 1))
    G.Nproj0 = int(Nproj)
    G.Nproj = G.osangles * int(Nproj)
    G.Nslices = int(Nslices)
    G.cor_f = float(cor)
    G.cor = int(cor)                       # params.cu:49 truncates to int
    G.cubic = (interp_type == 'cubic')
    G.proj = np.arange(0, G.Nproj) * np.pi / G.Nproj - G.beta / 2
    G.s = np.linspace(-1, 1, G.N)
    b = G.beta
    G.aR = np.sin(b / 2) / (1 + np.sin(b / 2))
    G.am = (np.cos(b / 2) - np.sin(b / 2)) / (1 + np.sin(b / 2))
    G.g = osg(G.aR, b / 2)
    G.Ntheta = G.N
    G.Nrho = 2 * G.N
    G.dtheta = (2 * b) / G.Ntheta
    G.drho = (G.g - np.log(G.am)) / G.Nrho
    G.thsp = (np.arange(-G.Ntheta / 2, G.Ntheta / 2) * np.float64(np.float32(G.dtheta))).astype(np.float32)
    G.rhosp = (np.arange(-G.Nrho, 0) * G.drho).astype(np.float32)
    return G


# --------------------------------------------------------------------------
# convolution kernels (initsfwd.py:69-93, initsadj.py:119-143)
# --------------------------------------------------------------------------
_CORRECTING = 1 + np.array([-216254335, 679543284, -1412947389, 2415881496, -3103579086,
                            2939942400, -2023224114, 984515304, -321455811, 63253516,
                            -5675265]) / 958003200.0


def fzeta(Ntheta, Nrho, betas, rhos, a, osthlarge, adjoint, mode='ref', chunk=256):
    """fzeta_loop_weights(_adj).  Returns the centred [Nrho, Ntheta] kernel (complex128).

    mode 'ref' follows the reference's dtypes: the angle grid and cos() are
    float32, pow/fft run in complex128 and each row is stored as complex64.
    mode 'fp64' evaluates everything in float64 and never rounds.
    """
    NL = osthlarge * Ntheta
    krho = np.arange(-Nrho / 2, Nrho / 2, dtype=np.float32)
    if mode == 'ref':
        thL = np.arange(-NL / 2, NL / 2, dtype=np.float32) / NL * betas
        h = np.ones(NL, dtype=np.float32)
    else:
        thL = np.arange(-NL / 2, NL / 2) / NL * betas
        h = np.ones(NL)
    corr = _CORRECTING.copy()
    corr[0] = 2 * (corr[0] - 0.5)
    h[0] = h[0] * corr[0]
    for j in range(1, len(corr)):
        h[j] = h[j] * corr[j]
        h[-1 - j + 1] = h[-1 - j + 1] * corr[j]
    cosL = np.cos(thL)
    lc = np.log(cosL.astype(np.float64))
    out = np.zeros((Nrho, Ntheta), dtype=np.complex128)
    for j0 in range(0, Nrho, chunk):
        kk = krho[j0:j0 + chunk]
        if mode == 'ref':
            rows = np.empty((len(kk), NL), dtype=np.complex128)
            for i, kj in enumerate(kk):
                if adjoint:
                    ex = 2 * np.pi * 1j * kj / rhos - a
                else:
                    ex = -2 * np.pi * 1j * kj / rhos - 1 - a
                rows[i] = h * pow(cosL, ex)
        else:
            kd = kk.astype(np.float64)
            ex = (2 * np.pi * 1j * kd / rhos - a) if adjoint else (-2 * np.pi * 1j * kd / rhos - 1 - a)
            rows = np.exp(ex[:, None] * lc[None, :]) * h[None, :]
        F = np.fft.fftshift(np.fft.fft(np.fft.fftshift(rows, axes=1), axis=1), axes=1)
        F = F[:, NL // 2 - Ntheta // 2:NL // 2 + Ntheta // 2]
        if mode == 'ref':
            F = F.astype(np.complex64)
        out[j0:j0 + chunk] = F
    if mode == 'ref':
        out = (out.astype(np.complex64) * (thL[1] - thL[0])).astype(np.complex128)
    else:
        out = out * (thL[1] - thL[0])
    out[0] = 0
    out[:, 0] = 0
    return out


# --------------------------------------------------------------------------
# FBP filter (initsadj.py:146-203)
# --------------------------------------------------------------------------
def wint(n, t):
    N = len(t)
    s = np.linspace(1e-40, 1, n)
    tmp1 = np.arange(n)
    tmp2 = np.arange(1, n + 2)
    iv = np.linalg.inv(np.exp(np.outer(tmp1, np.log(s))))
    u = np.diff(np.exp(np.outer(tmp2, np.log(s))) * np.tile(1.0 / tmp2[..., None], [1, n]))
    W1 = iv @ u[1:n + 1, :]
    W2 = iv @ u[0:n, :]
    p = 1 / np.concatenate((np.arange(1, n), (n - 1) * np.ones(N - 2 * (n - 1) - 1), np.arange(n - 1, 0, -1)))
    w = np.zeros(N)
    for j in range(N - n + 1):
        W = ((t[j + n - 1] - t[j]) ** 2) * W1 + (t[j + n - 1] - t[j]) * t[j] * W2
        for k in range(n - 1):
            w[j:j + n] = w[j:j + n] + p[j + k] * W[:, k]
    wn = w
    wn[-40:] = (w[-40]) / (N - 40) * np.arange(N - 40, N)
    return wn


FILTERS = ('ramp', 'shepp-logan', 'cosine', 'cosine2', 'hamming', 'hann', 'parzen')


def take_filter(N, name):
    """initsadj.py:146-173; returns the float64 filter of length 4N."""
    os_ = 4
    d = 0.5
    Ne = os_ * N
    t = np.arange(0, Ne / 2 + 1) / Ne
    w = Ne * 0.5 * wint(12, t)
    if name == 'ramp':
        wfa = w
    elif name == 'shepp-logan':
        wfa = w * np.sinc(t / (2 * d)) * (t / d <= 2)
    elif name == 'cosine':
        wfa = w * np.cos(np.pi * t / (2 * d)) * (t / d <= 1)
    elif name == 'cosine2':
        wfa = w * (np.cos(np.pi * t / (2 * d))) ** 2 * (t / d <= 1)
    elif name == 'hamming':
        wfa = w * (.54 + .46 * np.cos(np.pi * t / d)) * (t / d <= 1)
    elif name == 'hann':
        wfa = w * (1 + np.cos(np.pi * t / d)) / 2.0 * (t / d <= 1)
    elif name == 'parzen':
        wfa = w * pow(1 - t / d, 3) * (t / d <= 1)
    else:
        raise ValueError('unknown filter %r' % (name,))
    wfa = wfa * (wfa >= 0)
    mid = np.array([2 * wfa[0]])
    out = np.concatenate((np.flipud(wfa[1:]), mid, wfa[1:]))
    return out[:-1]


# --------------------------------------------------------------------------
# tables (initsfwd.py:15-66, initsadj.py:19-116)
#
# mode 'ref' repeats the reference's dtype flow (float32 grids, NumPy 2
# promotion: Python scalars are weak, NumPy scalars strong), so its index sets
# and values equal the reference precompute run with NumPy in place of CuPy.
# mode 'fp64' keeps the 'ref' index sets and evaluates every value in float64.
# --------------------------------------------------------------------------
def _span_pids(G, ang):
    b = G.beta
    return [np.where((ang >= k * b - b / 2) & (ang < k * b + b / 2))[0] for k in range(NSPAN)]


def _b3com(G, mode):
    if mode == 'ref':
        th, rh = G.thsp, G.rhosp
    else:
        th, rh = G.thsp.astype(np.float64), G.rhosp.astype(np.float64)
    B3th = np.fft.fft(np.fft.ifftshift(splineB3(th, 1)))
    B3rho = np.fft.fft(np.fft.ifftshift(splineB3(rh, 1)))
    return np.outer(B3rho, B3th).astype(np.complex128)


def fwd_tables(G, mode='ref'):
    """create_fwd: coordinates in texel units, fZ half spectrum [Nrho, Ntheta/2+1]."""
    b, aR = G.beta, G.aR
    T = {}

    def lp2c(tmp1, tmp2, k):
        c, sn = np.cos(k * b + b / 2), np.sin(k * b + b / 2)
        X = ((tmp1 - (1 - aR)) * c - tmp2 * sn) / aR
        Y = ((tmp1 - (1 - aR)) * sn + tmp2 * c) / aR
        Y *= (-1)
        return X, Y
    r1 = np.outer(np.exp(G.rhosp), np.cos(G.thsp)).ravel()      # float32, as the reference
    r2 = np.outer(np.exp(G.rhosp), np.sin(G.thsp)).ravel()
    if mode == 'ref':
        v1, v2 = r1, r2
    else:
        e = np.exp(G.rhosp.astype(np.float64))
        th = G.thsp.astype(np.float64)
        v1 = np.outer(e, np.cos(th)).ravel()
        v2 = np.outer(e, np.sin(th)).ravel()
    lp2C1, lp2C2 = [], []
    for k in range(NSPAN):
        X, Y = lp2c(r1, r2, k)
        cids = np.where((X ** 2 + Y ** 2) <= 1)[0]
        if mode != 'ref':
            X, Y = lp2c(v1, v2, k)
        lp2C1.append(X[cids])
        lp2C2.append(Y[cids])
    T['cids'] = cids
    s0, th0 = np.meshgrid(G.s, G.proj)
    th0 = th0.ravel()
    s0 = s0.ravel()
    T['pids'] = _span_pids(G, th0)
    p2lp1, p2lp2 = [], []
    for k in range(NSPAN):
        th00 = th0[T['pids'][k]] - k * b
        s00 = s0[T['pids'][k]]
        p2lp1.append(th00)
        p2lp2.append(np.log(s00 * aR + (1 - aR) * np.cos(th00)))
    T['lp2C1'] = [(x + 1) / 2 * (G.N - 1) for x in lp2C1]
    T['lp2C2'] = [(x + 1) / 2 * (G.N - 1) for x in lp2C2]
    T['p2lp1'] = [(x - G.thsp[0]) / (G.thsp[-1] - G.thsp[0]) * (G.Ntheta - 1) for x in p2lp1]
    T['p2lp2'] = [(x - G.rhosp[0]) / (G.rhosp[-1] - G.rhosp[0]) * (G.Nrho - 1) for x in p2lp2]
    const = np.sqrt(G.N * G.osangles / G.Nproj) * np.pi / 4 / aR / np.sqrt(2)
    fZ = np.fft.fftshift(fzeta(G.Ntheta, G.Nrho, 2 * b, G.g - np.log(G.am), 0, 4, False, mode))
    fZ = fZ[:, :G.Ntheta // 2 + 1] * const
    if G.cubic:
        fZ = fZ / _b3com(G, mode)[:, :G.Ntheta // 2 + 1]
    T['fZ'] = fZ
    return T


def adj_tables(G, filter_type, mode='ref'):
    """create_adj."""
    b, aR, am, g = G.beta, G.aR, G.am, G.g
    N = G.N
    T = {}
    x1, x2 = np.meshgrid(np.linspace(-1, 1, N), np.linspace(-1, 1, N))
    x1 = x1.ravel()
    x2 = x2.ravel()
    x2 = x2 * (-1)
    cids = np.where(x1 ** 2 + x2 ** 2 <= 1)[0]
    T['cids'] = cids
    C2lp1, C2lp2 = [], []
    for k in range(NSPAN):
        z1 = aR * (x1[cids] * np.cos(k * b + b / 2) + x2[cids] * np.sin(k * b + b / 2)) + (1 - aR)
        z2 = aR * (-x1[cids] * np.sin(k * b + b / 2) + x2[cids] * np.cos(k * b + b / 2))
        C2lp1.append(np.arctan2(z2, z1))
        C2lp2.append(np.log(np.sqrt(z1 ** 2 + z2 ** 2)))

    def polar(z1, z2):
        """log-polar -> polar coordinates and the wrap sets (initsadj.py:41-72)."""
        z1 = z1.ravel()
        z2 = z2.ravel()
        z2n = z2 - (1 - aR) * np.cos(z1)
        z2n = z2n / aR
        lpids = np.where((z1 >= -b / 2) & (z1 < b / 2) & (abs(z2n) <= 1))[0]
        wids = np.where(np.log(z2) > +g)[0]
        z2nw = np.exp(np.log(z2[wids]) + np.log(am) - g) - (1 - aR) * np.cos(z1[wids])
        z2nw = z2nw / aR
        lw = np.where((z1[wids] >= -b / 2) & (z1[wids] < b / 2) & (abs(z2nw) <= 1))[0]
        wids2 = np.where(np.log(z2) < np.log(am) - g + (G.rhosp[1] - G.rhosp[0]))[0]
        z2nw2 = np.exp(np.log(z2[wids2]) - np.log(am) + g) - (1 - aR) * np.cos(z1[wids2])
        z2nw2 = z2nw2 / aR
        lw2 = np.where((z1[wids2] >= -b / 2) & (z1[wids2] < b / 2) & (abs(z2nw2) <= 1))[0]
        return z1, z2n, lpids, wids, z2nw, lw, wids2, z2nw2, lw2
    z1, z2 = np.meshgrid(G.thsp, np.exp(G.rhosp))                # float32, as the reference
    z1, z2n, lpids, wids, z2nw, lw, wids2, z2nw2, lw2 = polar(z1, z2)
    if mode != 'ref':
        z1, z2 = np.meshgrid(G.thsp.astype(np.float64), np.exp(G.rhosp.astype(np.float64)))
        z1, z2n, _, _, z2nw, _, _, z2nw2, _ = polar(z1, z2)
        # keep the 'ref' index sets; re-evaluate the wrap values at them
        zz1 = z1
        z2f = z2.ravel()
        z2nw = (np.exp(np.log(z2f[wids]) + np.log(am) - g) - (1 - aR) * np.cos(zz1[wids])) / aR
        z2nw2 = (np.exp(np.log(z2f[wids2]) - np.log(am) + g) - (1 - aR) * np.cos(zz1[wids2])) / aR
    T['lpids'] = lpids
    lp2p1 = [(z1[lpids] + k * b) for k in range(NSPAN)]
    lp2p2 = [z2n[lpids] for k in range(NSPAN)]
    # initsadj.py:69 indexes z1 by positions inside the wrap subsets; the wrap
    # subsets are whole grid rows starting at a row boundary, so this equals z1
    # at the wrap points themselves.  Restated literally.
    sel = np.concatenate((lw, lw2))
    lp2p1w = [(z1[sel] + k * b) for k in range(NSPAN)]
    lp2p2w = [np.concatenate((z2nw[lw], z2nw2[lw2])) for k in range(NSPAN)]
    T['wids'] = np.concatenate((wids[lw], wids2[lw2]))
    pids = _span_pids(G, G.proj)
    proj0 = [G.proj[p[0]] for p in pids]
    projl = [G.proj[p[-1]] - G.proj[p[0]] for p in pids]
    projp = (G.Nproj - 1) / (proj0[NSPAN - 1] + projl[NSPAN - 1] - proj0[0])
    T['lp2p1'] = [(lp2p1[k] - proj0[k]) / projl[k] * (len(pids[k]) - 1) + (proj0[k] - proj0[0]) * projp
                  for k in range(NSPAN)]
    T['lp2p1w'] = [(lp2p1w[k] - proj0[k]) / projl[k] * (len(pids[k]) - 1) + (proj0[k] - proj0[0]) * projp
                   for k in range(NSPAN)]
    T['lp2p2'] = [(x + 1) / 2 * (N - 1) for x in lp2p2]
    T['lp2p2w'] = [(x + 1) / 2 * (N - 1) for x in lp2p2w]
    T['C2lp1'] = [(x - G.thsp[0]) / (G.thsp[-1] - G.thsp[0]) * (G.Ntheta - 1) for x in C2lp1]
    T['C2lp2'] = [(x - G.rhosp[0]) / (G.rhosp[-1] - G.rhosp[0]) * (G.Nrho - 1) for x in C2lp2]
    const = (N + 1) * (N - 1) / N ** 2 / 2 * np.sqrt(G.osangles * G.Nproj / N / 2)
    fZ = np.fft.fftshift(fzeta(G.Ntheta, G.Nrho, 2 * b, g - np.log(am), 0, 4, True, mode))
    fZ = fZ[:, :G.Ntheta // 2 + 1] * const
    if G.cubic:
        fZ = fZ / _b3com(G, mode)[:, :G.Ntheta // 2 + 1]
    T['fZ'] = fZ
    T['filter'] = None if filter_type in (None, 'none') else take_filter(N, filter_type)
    for k in ('lp2C1', 'lp2C2', 'C2lp1', 'C2lp2', 'lp2p1', 'lp2p2', 'lp2p1w', 'lp2p2w'):
        if k in T:
            T[k] = [np.asarray(x, dtype=np.float64) for x in T[k]]
    return T


_FLOAT_KEYS = ('lp2C1', 'lp2C2', 'p2lp1', 'p2lp2', 'C2lp1', 'C2lp2', 'lp2p1', 'lp2p2', 'lp2p1w', 'lp2p2w')


def round_tables(T):
    """Round a table dict once to the float32/complex64 values the GPU receives."""
    R = {}
    for k, v in T.items():
        if k in _FLOAT_KEYS:
            R[k] = [np.float32(x).astype(np.float64) for x in v]
        elif k == 'fZ':
            R[k] = v.astype(np.complex64).astype(np.complex128)
        elif k == 'filter':
            R[k] = None if v is None else v.astype(np.float32).astype(np.float64)
        else:
            R[k] = v
    return R


def erho_table(G, mode='ref'):
    """initsgl.py:44: e^rho per log-polar row (float32 exp in the reference)."""
    if mode == 'ref':
        return np.exp(G.rhosp).astype(np.float64)
    return np.exp(G.rhosp.astype(np.float64))


# --------------------------------------------------------------------------
# packed parameter arrays (initsgl.py:55-56, initsfwd.py:96-126,
# initsadj.py:205-244; read back as in params.cu:40-145)
# --------------------------------------------------------------------------
def _fzvec(fZ):
    v = np.zeros(fZ.size * 2, dtype=np.float32)
    v[::2] = fZ.real.ravel()
    v[1::2] = fZ.imag.ravel()
    return v


def pack_params(G, Tf, Ta, erho):
    """Return (glpars, fwdparsi, fwdparamsf, adjparsi, adjparamsf) in the reference layout."""
    head = np.array([G.N, G.N0, G.Ntheta, G.Nrho, NSPAN, G.Nproj, G.Nslices, G.cor_f,
                     G.osangles, G.cubic], dtype=np.float32)
    glpars = np.concatenate((head, np.repeat(np.float32(erho), G.Ntheta)))
    fi = ff = None
    if Tf:
        fi = np.concatenate([[len(p) for p in Tf['pids']]] + list(Tf['pids'])
                            + [[len(Tf['cids'])], Tf['cids']]).astype(np.int32)
        ff = np.concatenate(list(Tf['lp2C1']) + list(Tf['lp2C2']) + list(Tf['p2lp1'])
                            + list(Tf['p2lp2']) + [_fzvec(Tf['fZ'])]).astype(np.float32)
    ai = [[len(Ta['cids'])], [len(Ta['lpids'])], [len(Ta['wids'])], Ta['cids'], Ta['lpids'], Ta['wids']]
    af = (list(Ta['C2lp1']) + list(Ta['C2lp2']) + list(Ta['lp2p1']) + list(Ta['lp2p2'])
          + list(Ta['lp2p1w']) + list(Ta['lp2p2w']) + [_fzvec(Ta['fZ'])])
    if Ta.get('filter') is not None:
        af.append(np.float32(Ta['filter']))
        ai.append([1])
    else:
        ai.append([0])
    ai = np.concatenate(ai).astype(np.int32)
    af = np.concatenate(af).astype(np.float32)
    return glpars, fi, ff, ai, af


def unpack_params(glpars, fi, ff, ai, af):
    """Parse packed arrays into (Geometry, Tf, Ta, erho) with float64 values."""
    g = np.asarray(glpars)
    G = Geometry()
    G.N, G.N0, G.Ntheta, G.Nrho, nspan, G.Nproj, G.Nslices = [int(x) for x in g[:7]]
    assert nspan == NSPAN
    G.cor_f = float(g[7])
    G.cor = int(g[7])
    G.osangles = int(g[8])
    G.cubic = bool(int(g[9]))
    G.Nproj0 = G.Nproj // G.osangles
    G.beta = np.pi / NSPAN
    erho = np.asarray(g[10:10 + G.Nrho * G.Ntheta], dtype=np.float64).reshape(G.Nrho, G.Ntheta)[:, 0].copy()
    nh = G.Ntheta // 2 + 1

    def fz(v):
        v = np.asarray(v, dtype=np.float64)
        return (v[::2] + 1j * v[1::2]).reshape(G.Nrho, nh)
    Tf = {}
    if fi is not None:
        fi = np.asarray(fi)
        ff = np.asarray(ff, dtype=np.float64)
        npids = [int(x) for x in fi[:NSPAN]]
        o = NSPAN
        Tf['pids'] = []
        for k in range(NSPAN):
            Tf['pids'].append(fi[o:o + npids[k]].astype(np.int64))
            o += npids[k]
        nc = int(fi[o])
        Tf['cids'] = fi[o + 1:o + 1 + nc].astype(np.int64)
        o = 0
        for key, n in (('lp2C1', [nc] * 3), ('lp2C2', [nc] * 3), ('p2lp1', npids), ('p2lp2', npids)):
            Tf[key] = []
            for k in range(NSPAN):
                Tf[key].append(ff[o:o + n[k]])
                o += n[k]
        Tf['fZ'] = fz(ff[o:o + 2 * G.Nrho * nh])
    ai = np.asarray(ai)
    af = np.asarray(af, dtype=np.float64)
    nc, nl, nw = [int(x) for x in ai[:3]]
    Ta = {'cids': ai[3:3 + nc].astype(np.int64),
          'lpids': ai[3 + nc:3 + nc + nl].astype(np.int64),
          'wids': ai[3 + nc + nl:3 + nc + nl + nw].astype(np.int64)}
    flag = int(ai[3 + nc + nl + nw])
    o = 0
    for key, n in (('C2lp1', nc), ('C2lp2', nc), ('lp2p1', nl), ('lp2p2', nl), ('lp2p1w', nw), ('lp2p2w', nw)):
        Ta[key] = []
        for k in range(NSPAN):
            Ta[key].append(af[o:o + n])
            o += n
    Ta['fZ'] = fz(af[o:o + 2 * G.Nrho * nh])
    o += 2 * G.Nrho * nh
    Ta['filter'] = af[o:o + 4 * G.N].copy() if flag == 1 else None
    return G, Tf, Ta, erho


# --------------------------------------------------------------------------
# cubic B-spline prefilter (main_kernels.cuh:97-185, lpRgpu.cu:219-240)
# --------------------------------------------------------------------------
def prefilter_lines(x, axis):
    """ConvertToInterpolationCoefficients along ``axis`` (in float64, returns a copy)."""
    c = np.moveaxis(np.array(x, dtype=np.float64), axis, 0).copy()
    L = c.shape[0]
    z = POLE
    # InitialCausalCoefficient: c[0] counted once up front and again at n=0
    hor = min(12, L)
    s = c[0].copy()
    zn = z
    for n in range(hor):
        s += zn * c[n]
        zn *= z
    c[0] = LAMBDA * s
    for n in range(1, L):
        c[n] = LAMBDA * c[n] + z * c[n - 1]
    c[L - 1] = (z / (z - 1.0)) * c[L - 1]
    for n in range(L - 2, -1, -1):
        c[n] = z * (c[n + 1] - c[n])
    return np.moveaxis(c, 0, axis)


def prefilter2d(x):
    """Rows (along x) first, then columns (along y), as prefilter2D does."""
    return prefilter_lines(prefilter_lines(x, -1), -2)


# --------------------------------------------------------------------------
# interpolation with wrap addressing (main_kernels.cuh:9-84)
# --------------------------------------------------------------------------
def bspline_weights(f):
    one = 1.0 - f
    return [one ** 3 / 6.0,
            2.0 / 3.0 - 0.5 * f * f * (2.0 - f),
            2.0 / 3.0 - 0.5 * one * one * (2.0 - one),
            f ** 3 / 6.0]


def interp2d(img, x, y, cubic, tex8=False):
    """Sample img[S, H, W] at texel-index positions (x along W, y along H).

    ``interp`` samples the texture at (x+0.5, y+0.5) in texel units, i.e. at
    index position (x, y) with wrap addressing on both axes.  The cubic mode is
    the tensor-product cubic B-spline, which the reference builds from four
    bilinear fetches; ``tex8`` quantises bilinear fractions to 1/256 the way
    texture hardware does (only meaningful for comparison).
    """
    S, H, W = img.shape
    flat = img.reshape(S, H * W)
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    ix = np.floor(x)
    iy = np.floor(y)
    fx = x - ix
    fy = y - iy
    ix = ix.astype(np.int64)
    iy = iy.astype(np.int64)
    out = np.zeros((S, x.size))
    if cubic and not tex8:
        wx = bspline_weights(fx)
        wy = bspline_weights(fy)
        for j in range(4):
            row = np.mod(iy + j - 1, H) * W
            acc = np.zeros((S, x.size))
            for i in range(4):
                acc += wx[i] * flat[:, row + np.mod(ix + i - 1, W)]
            out += wy[j] * acc
        return out
    if cubic and tex8:
        wx = bspline_weights(fx)
        wy = bspline_weights(fy)
        g0x, g1x = wx[0] + wx[1], wx[2] + wx[3]
        g0y, g1y = wy[0] + wy[1], wy[2] + wy[3]
        h0x = wx[1] / g0x - 1 + ix      # index-space positions of the 4 fetches
        h1x = wx[3] / g1x + 1 + ix
        h0y = wy[1] / g0y - 1 + iy
        h1y = wy[3] / g1y + 1 + iy

        def lin(px, py):
            return _linear_fetch(flat, H, W, px, py, True)
        t00, t10 = lin(h0x, h0y), lin(h1x, h0y)
        t01, t11 = lin(h0x, h1y), lin(h1x, h1y)
        a = g0y * t00 + g1y * t01
        b = g0y * t10 + g1y * t11
        return g0x * a + g1x * b
    return _linear_fetch(flat, H, W, x, y, tex8)


def _linear_fetch(flat, H, W, x, y, tex8):
    ix = np.floor(x)
    iy = np.floor(y)
    fx = x - ix
    fy = y - iy
    if tex8:
        fx = np.round(fx * 256.0) / 256.0
        fy = np.round(fy * 256.0) / 256.0
    ix = ix.astype(np.int64)
    iy = iy.astype(np.int64)
    r0 = np.mod(iy, H) * W
    r1 = np.mod(iy + 1, H) * W
    c0 = np.mod(ix, W)
    c1 = np.mod(ix + 1, W)
    return ((1 - fy) * ((1 - fx) * flat[:, r0 + c0] + fx * flat[:, r0 + c1])
            + fy * ((1 - fx) * flat[:, r1 + c0] + fx * flat[:, r1 + c1]))


# --------------------------------------------------------------------------
# log-polar convolution (lpRgpu.cu:270-277, simple_kernels.cuh:2-12)
# --------------------------------------------------------------------------
def lp_conv(G, grid, fZ):
    """cuFFT 2-D R2C over (Nrho, Ntheta), multiply by fZ/(Nrho*Ntheta), C2R."""
    X = np.fft.rfft2(grid, axes=(-2, -1))
    X *= fZ[None]
    return np.fft.irfft2(X, s=(G.Nrho, G.Ntheta), axes=(-2, -1))


# --------------------------------------------------------------------------
# pipelines (lpRgpu.cu:243-330)
# --------------------------------------------------------------------------
def fwd_span(G, T, fp, erho, k, tex8=False):
    """One span of execFwd (lpRgpu.cu:257-285) on the prefiltered image fp[S, N, N]:
    returns that span's values at its polar points pids[k] (shape [S, len(pids[k])])."""
    S = fp.shape[0]
    dfl = np.zeros((S, G.Nrho * G.Ntheta))
    dfl[:, T['cids']] = interp2d(fp, T['lp2C1'][k], T['lp2C2'][k], G.cubic, tex8)
    dfl = dfl.reshape(S, G.Nrho, G.Ntheta) * erho[None, :, None]
    dfl = lp_conv(G, dfl, T['fZ'])
    return interp2d(dfl, T['p2lp1'][k], T['p2lp2'][k], G.cubic, tex8)


def fwd_core(G, T, f, erho, tex8=False):
    """execFwd on the padded image f[S, N, N]; returns R[S, Nproj, N] (internal angles)."""
    S = f.shape[0]
    N = G.N
    fp = prefilter2d(f) if G.cubic else np.asarray(f, dtype=np.float64)
    R = np.zeros((S, G.Nproj * N))
    for k in range(NSPAN):
        R[:, T['pids'][k]] += fwd_span(G, T, fp, erho, k, tex8)
    return R.reshape(S, G.Nproj, N)


def adj_span(G, T, Rp, k, tex8=False):
    """One span of execAdj (lpRgpu.cu:302-329) on the prefiltered sinogram Rp[S, Nproj, N]:
    returns that span's contribution at the disk pixels cids (shape [S, len(cids)])."""
    S = Rp.shape[0]
    dfl = np.zeros((S, G.Nrho * G.Ntheta))
    dfl[:, T['lpids']] += interp2d(Rp, T['lp2p2'][k], T['lp2p1'][k], G.cubic, tex8)
    if len(T['wids']):
        dfl[:, T['wids']] += interp2d(Rp, T['lp2p2w'][k], T['lp2p1w'][k], G.cubic, tex8)
    dfl = lp_conv(G, dfl.reshape(S, G.Nrho, G.Ntheta), T['fZ'])
    return interp2d(dfl, T['C2lp1'][k], T['C2lp2'][k], G.cubic, tex8)


def adj_core(G, T, R, tex8=False):
    """execAdj on the internal sinogram R[S, Nproj, N]; returns f[S, N, N]."""
    S = R.shape[0]
    N = G.N
    Rp = prefilter2d(R) if G.cubic else np.asarray(R, dtype=np.float64)
    f = np.zeros((S, N * N))
    for k in range(NSPAN):
        f[:, T['cids']] += adj_span(G, T, Rp, k, tex8)
    return f.reshape(S, N, N)


def apply_filter(G, R, filt):
    """applyFilter (lpRgpu.cu:333-382), restated step by step per slice."""
    S, P, N = R.shape
    M = 4 * N
    off = M // 2 - N // 2
    tx = np.arange(M)
    ty = np.arange(P)
    sgn = np.outer(1 - 2 * ((ty + 1) % 2), 1 - 2 * ((tx + 1) % 2)).astype(np.float64)
    out = np.empty_like(R, dtype=np.float64)
    for s in range(S):
        c = np.zeros((P, M), dtype=np.complex128)
        c[:, off:off + N] = R[s]
        c *= sgn
        c = np.fft.fft(c, axis=1)
        c *= sgn
        c *= filt[None, :]
        c *= sgn
        c = np.fft.ifft(c, axis=1) * M
        c *= sgn
        out[s] = c[:, off:off + N].real / M
    return out


def fwd(G, T, f_in, erho=None, tex8=False):
    """execFwdManyPtr (lpRgpu.cu:184-193): f_in[S0, N0, N0] -> R[S0, Nproj0, N0]."""
    if erho is None:
        erho = erho_table(G)
    S0 = f_in.shape[0]
    N, N0 = G.N, G.N0
    o = N // 2 - N0 // 2
    df = np.zeros((S0, N, N))
    df[:, o:o + N0, o:o + N0] = f_in
    R = fwd_core(G, T, df, erho, tex8)
    c0 = N // 2 - G.cor
    return R[:, ::G.osangles, c0:c0 + N0][:, :G.Nproj0]


def pad_sinogram(G, R_in):
    """copy3Dshifted + stepangles + padker (lpRgpu.cu:199-203, :211-216)."""
    S0 = R_in.shape[0]
    N, N0 = G.N, G.N0
    c0 = N // 2 - G.cor
    dR = np.zeros((S0, G.Nproj, N))
    dR[:, ::G.osangles, c0:c0 + N0] = R_in
    lb, rb = N // 2 - G.cor, N // 2 + N0 - G.cor - 1
    if lb > 0:
        dR[:, :, :lb] = dR[:, :, lb:lb + 1]
    if rb < N - 1:
        dR[:, :, rb + 1:] = dR[:, :, rb:rb + 1]
    return dR


def adj(G, T, R_in, tex8=False):
    """execAdjManyPtr (lpRgpu.cu:196-207): R_in[S0, Nproj0, N0] -> f[S0, N0, N0]."""
    N, N0 = G.N, G.N0
    dR = pad_sinogram(G, R_in)
    if T.get('filter') is not None:
        dR = apply_filter(G, dR, T['filter'])
    f = adj_core(G, T, dR, tex8)
    o = N // 2 - N0 // 2
    return f[:, o:o + N0, o:o + N0]


class Transform:
    """Geometry plus tables, with fwd/adj on host arrays.

    mode 'ref' builds the tables the way the reference does; mode 'fp64'
    keeps the same index sets with float64 values.  ``rounded`` rounds the
    values once to float32/complex64 (what the GPU receives).  ``tables`` may
    supply (Tf, Ta, erho) directly, e.g. parsed from packed parameter arrays.
    """

    def __init__(self, N0, Nproj, Nslices=1, filter_type='none', cor=None, interp_type='cubic',
                 mode='ref', rounded=True, fwd=True, tables=None):
        if cor is None:
            cor = N0 / 2
        self.G = create_geometry(N0, Nproj, Nslices, cor, interp_type)
        if tables is not None:
            self.Tf, self.Ta, self.erho = tables
            return
        Tf = fwd_tables(self.G, mode) if fwd else {}
        Ta = adj_tables(self.G, filter_type, mode)
        if rounded:
            Tf = round_tables(Tf) if fwd else {}
            Ta = round_tables(Ta)
        self.Tf, self.Ta = Tf, Ta
        e = erho_table(self.G, mode)
        self.erho = np.float32(e).astype(np.float64) if rounded else e

    @classmethod
    def from_packed(cls, glpars, fi, ff, ai, af):
        G, Tf, Ta, erho = unpack_params(glpars, fi, ff, ai, af)
        self = cls.__new__(cls)
        self.G, self.Tf, self.Ta, self.erho = G, Tf, Ta, erho
        return self

    def packed(self):
        return pack_params(self.G, self.Tf, self.Ta, self.erho)

    def fwd(self, f):
        return fwd(self.G, self.Tf, np.asarray(f, dtype=np.float64), self.erho)

    def adj(self, R):
        return adj(self.G, self.Ta, np.asarray(R, dtype=np.float64))

    def fwd_T(self, R):
        """Exact transpose of fwd (gradient of <fwd(f), R> with respect to f)."""
        return fwd_T(self.G, self.Tf, np.asarray(R, dtype=np.float64), self.erho)


# --------------------------------------------------------------------------
# exact transpose of the forward operator (for the autograd backward); this
# is NOT the reference's adjoint, which is a different discretisation
# --------------------------------------------------------------------------
def prefilter_lines_T(y, axis):
    """Transpose of prefilter_lines along `axis` (main_kernels.cuh:97-142 as a matrix)."""
    c = np.moveaxis(np.array(y, dtype=np.float64), axis, 0).copy()
    L = c.shape[0]
    z = POLE
    q = z / (z - 1.0)
    # A^T: causal sum t[m] = y[m] + z t[m-1]; a[m] = -z t[m], a[L-1] = q t[L-1]
    t = c[0].copy()
    a = np.empty_like(c)
    for m in range(L):
        if m > 0:
            t = c[m] + z * t
        a[m] = -z * t if m < L - 1 else q * t
    # anticausal sum w[m] = a[m] + z w[m+1]
    w = np.empty_like(c)
    w[L - 1] = a[L - 1]
    for m in range(L - 2, -1, -1):
        w[m] = a[m] + z * w[m + 1]
    # K^T: Lambda (w[m] + [m < H] z^(m+1) w[0])
    hor = min(12, L)
    out = LAMBDA * w
    for m in range(hor):
        out[m] += LAMBDA * z ** (m + 1) * w[0]
    return np.moveaxis(out, 0, axis)


def prefilter2d_T(y):
    return prefilter_lines_T(prefilter_lines_T(y, -2), -1)


def interp2d_T(shape, vals, x, y, cubic):
    """Transpose of interp2d: scatter vals[S, Np] into an image of `shape` = (S, H, W)."""
    S, H, W = shape
    vals = np.asarray(vals, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    ix = np.floor(x)
    iy = np.floor(y)
    fx = x - ix
    fy = y - iy
    ix = ix.astype(np.int64)
    iy = iy.astype(np.int64)
    out = np.zeros((S, H * W))
    if cubic:
        wx = bspline_weights(fx)
        wy = bspline_weights(fy)
        taps = [(j - 1, i - 1, wy[j] * wx[i]) for j in range(4) for i in range(4)]
    else:
        taps = [(0, 0, (1 - fy) * (1 - fx)), (0, 1, (1 - fy) * fx), (1, 0, fy * (1 - fx)), (1, 1, fy * fx)]
    for dj, di, wgt in taps:
        idx = np.mod(iy + dj, H) * W + np.mod(ix + di, W)
        for s in range(S):
            out[s] += np.bincount(idx, weights=wgt * vals[s], minlength=H * W)
    return out.reshape(S, H, W)


def fwd_T(G, T, R_out, erho):
    """Exact transpose of fwd(): R_out[S0, Nproj0, N0] -> f[S0, N0, N0]."""
    S = R_out.shape[0]
    N, N0 = G.N, G.N0
    c0 = N // 2 - G.cor
    R = np.zeros((S, G.Nproj, N))
    R[:, ::G.osangles, c0:c0 + N0] = R_out
    Rf = R.reshape(S, -1)
    f = np.zeros((S, N, N))
    for k in range(NSPAN):
        H = interp2d_T((S, G.Nrho, G.Ntheta), Rf[:, T['pids'][k]], T['p2lp1'][k], T['p2lp2'][k], G.cubic)
        X = np.fft.rfft2(H, axes=(-2, -1)) * np.conj(T['fZ'])[None]
        H = np.fft.irfft2(X, s=(G.Nrho, G.Ntheta), axes=(-2, -1)) * erho[None, :, None]
        f += interp2d_T((S, N, N), H.reshape(S, -1)[:, T['cids']], T['lp2C1'][k], T['lp2C2'][k], G.cubic)
    if G.cubic:
        f = prefilter2d_T(f)
    o = N // 2 - N0 // 2
    return f[:, o:o + N0, o:o + N0]


# --------------------------------------------------------------------------
# solvers (lpmethods.py), float64, used to check the GPU solvers
# --------------------------------------------------------------------------
def solve_fbp(tr, init, tomo, num_iter=0, reg_par=0):
    return tr.adj(tomo)


def solve_grad(tr, init, tomo, num_iter, reg_par):
    recon = np.array(init, dtype=np.float64)
    recon0 = recon
    grad0 = recon * 0
    S = tomo.shape[0]
    for i in range(num_iter):
        g = tr.fwd(recon)
        grad = tr.adj(2 * (g - tomo))
        if reg_par < 0:
            if i == 0:
                lam = 1e-3 * np.ones(S)
            else:
                lam = (np.sum((recon - recon0) * (grad - grad0), axis=(1, 2))
                       / np.sum((grad - grad0) * (grad - grad0), axis=(1, 2)))
        else:
            lam = reg_par * np.ones(S)
        recon0 = recon.copy()
        grad0 = grad.copy()
        recon = recon - lam[:, None, None] * grad
    return recon


def solve_cg(tr, init, tomo, num_iter, reg_par=0):
    recon = np.array(init, dtype=np.float64)
    b = tr.adj(tomo)
    f = tr.adj(tr.fwd(recon))
    r = b - f
    p = r.copy()
    rsold = np.sum(r * r)
    for i in range(num_iter):
        f = tr.adj(tr.fwd(p))
        alpha = rsold / np.sum(p * f)
        recon = recon + alpha * p
        r = r - alpha * f
        rsnew = np.sum(r * r)
        p = r + (rsnew / rsold) * p
        rsold = rsnew
    return recon


def solve_em(tr, init, tomo, num_iter, reg_par):
    recon = np.array(init, dtype=np.float64)
    xi = tr.adj(tomo * 0 + 1) + 1e-5
    for i in range(num_iter):
        g = tr.fwd(recon)
        upd = tr.adj(tomo / (g + np.float32(reg_par)))
        recon = recon * (upd / xi)
    return recon


def _tv_family(tr, init, tomo, num_iter, reg_par, prox):
    recon = np.array(init, dtype=np.float64)
    recon0 = recon
    prox0x = recon * 0
    prox0y = recon * 0
    div0 = recon * 0
    prox1 = tomo * 0.0
    lam = reg_par
    c = 0.35
    for i in range(num_iter):
        prox0x[:, :, :-1] += c * (recon[:, :, 1:] - recon[:, :, :-1])
        prox0y[:, :-1, :] += c * (recon[:, 1:, :] - recon[:, :-1, :])
        nprox = np.maximum(1, np.sqrt(prox0x * prox0x + prox0y * prox0y) / lam)
        prox0x = prox0x / nprox
        prox0y = prox0y / nprox
        g = tr.fwd(recon)
        prox1 = prox(prox1, g, c)
        recon = recon0
        div0[:, :, 1:] = (prox0x[:, :, 1:] - prox0x[:, :, :-1])
        div0[:, :, 0] = prox0x[:, :, 0]
        div0[:, 1:, :] += (prox0y[:, 1:, :] - prox0y[:, :-1, :])
        div0[:, 0, :] += prox0y[:, 0, :]
        p = tr.adj(prox1)
        recon0 = recon0 - c * p + c * div0
        recon = 2 * recon0 - recon
    return recon


def solve_tv(tr, init, tomo, num_iter, reg_par):
    return _tv_family(tr, init, tomo, num_iter, reg_par,
                      lambda p1, g, c: (p1 + c * g - c * tomo) / (1 + c))


def solve_tve(tr, init, tomo, num_iter, reg_par):
    def prox(p1, g, c):
        tmp = 0.5 * (p1 + c * g - 1 + np.sqrt((p1 + c * g - 1) ** 2 + 4 * c * tomo))
        tmp[tmp < 0] = 0
        return p1 + c * g - tmp
    return _tv_family(tr, init, tomo, num_iter, reg_par, prox)


def solve_tvl1(tr, init, tomo, num_iter, reg_par):
    def prox(p1, g, c):
        tmp = p1 + c * g - c * tomo
        tmp2 = np.abs(tmp) - 1
        tmp2[tmp2 < 0] = 0
        return tmp - tmp2 * np.sign(tmp)
    return _tv_family(tr, init, tomo, num_iter, reg_par, prox)


# --------------------------------------------------------------------------
# test data
# --------------------------------------------------------------------------
def ellipse_phantom(N, n_ellipses, rng):
    """Random-ellipse phantom on the reference grid linspace(-1,1,N) with the y flip."""
    x1, x2 = np.meshgrid(np.linspace(-1, 1, N), np.linspace(-1, 1, N))
    x2 = -x2
    img = np.zeros((N, N))
    for _ in range(n_ellipses):
        r = 0.7 * np.sqrt(rng.uniform())
        phi = 2 * np.pi * rng.uniform()
        cx, cy = r * np.cos(phi), r * np.sin(phi)
        a, b = rng.uniform(0.05, 0.35, size=2)
        rot = rng.uniform(0, np.pi)
        val = rng.uniform(-0.2, 1.0)
        u = (x1 - cx) * np.cos(rot) + (x2 - cy) * np.sin(rot)
        v = -(x1 - cx) * np.sin(rot) + (x2 - cy) * np.cos(rot)
        img[(u / a) ** 2 + (v / b) ** 2 <= 1] += val
    return img


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
