"""Second, independent restatement of the reference in numpy (test infrastructure only).

It follows the MATLAB source statement by statement (flips, permutes,
meshgrid, find, accumarray) rather than the reduced index formulas of
genfire_oracle.c, so the two restatements check each other.  It is meant
for small sizes only.  FP32 steps use numpy float32 arithmetic, which is
evaluated element-wise without fused multiply-add.
"""
import numpy as np


def mround(x):
    """MATLAB round: half away from zero."""
    x = np.asarray(x, dtype=np.float64)
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def quat_rot(vector, theta):
    """fillInFourierGrid_DFT.m:353-363."""
    theta = theta * np.pi / 180
    v = np.asarray(vector, dtype=np.float64)
    v = v / np.sqrt(np.dot(v, v))
    w = np.cos(theta / 2)
    x, y, z = (-np.sin(theta / 2) * v[0], -np.sin(theta / 2) * v[1], -np.sin(theta / 2) * v[2])
    return np.array([[1 - 2 * y ** 2 - 2 * z ** 2, 2 * x * y + 2 * w * z, 2 * x * z - 2 * w * y],
                     [2 * x * y - 2 * w * z, 1 - 2 * x ** 2 - 2 * z ** 2, 2 * y * z + 2 * w * x],
                     [2 * x * z + 2 * w * y, 2 * y * z - 2 * w * x, 1 - 2 * x ** 2 - 2 * y ** 2]])


def rotmat(v1, v2, v3, phi, theta, psi):
    return quat_rot(v1, phi) @ quat_rot(v2, theta) @ quat_rot(v3, psi)


def lu_solve_f32(R, B):
    """R \\ B in float32 by LU with partial pivoting (getf2 order), vectorised over columns."""
    A = np.array(R, dtype=np.float32)
    piv = []
    for k in range(3):
        p = k + int(np.argmax(np.abs(A[k:, k])))
        piv.append(p)
        if p != k:
            A[[k, p], :] = A[[p, k], :]
        if A[k, k] != 0 and k < 2:
            r = np.float32(1.0) / A[k, k]
            A[k + 1:, k] = A[k + 1:, k] * r
        for j in range(k + 1, 3):
            for i in range(k + 1, 3):
                A[i, j] = A[i, j] - A[i, k] * A[k, j]
    b = [np.array(B[i], dtype=np.float32) for i in range(3)]
    for k in range(3):
        if piv[k] != k:
            b[k], b[piv[k]] = b[piv[k]], b[k]
    for k in range(3):
        for i in range(k + 1, 3):
            b[i] = b[i] - b[k] * A[i, k]
    for k in range(2, -1, -1):
        b[k] = b[k] / A[k, k]
        for i in range(k):
            b[i] = b[i] - b[k] * A[i, k]
    return np.stack(b)


def half_grid(n1, n2, centro):
    """fillInFourierGrid_DFT.m:122-144: K1, K2, K3 flattened column-major."""
    if centro:
        k1 = np.arange(-(n1 // 2), 1, dtype=np.float32)
        k2 = np.arange(-(n2 // 2), n2 // 2 + 1, dtype=np.float32)
        k3 = np.arange(-(n1 // 2), n1 // 2 + 1, dtype=np.float32)
    else:
        k1 = np.arange(-int(np.ceil((n1 - 1) / 2)), int(np.floor((n1 - 1) / 2)) + 1, dtype=np.float32)
        k2 = np.arange(-int(np.ceil((n2 - 1) / 2)), int(np.floor((n2 - 1) / 2)) + 1, dtype=np.float32)
        k3 = k1
    K1, K2, K3 = np.meshgrid(k1, k2, k3, indexing="ij")
    return (K1.reshape(-1, order="F"), K2.reshape(-1, order="F"), K3.reshape(-1, order="F"),
            (k1.size, k2.size, k3.size))


def select(n1, n2, centro, cutoff, R32, nrm32):
    """Per-projection K-point selection (fillInFourierGrid_DFT.m:175-192)."""
    K1, K2, K3, _ = half_grid(n1, n2, centro)
    n = np.asarray(nrm32, dtype=np.float32)
    nn = np.sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2])
    h = n / nn
    D = np.abs(K1 * h[0] + K2 * h[1] + K3 * h[2])
    Dind = np.nonzero(D.astype(np.float64) < cutoff)[0]
    p1, p2, p3 = K1[Dind], K2[Dind], K3[Dind]
    s = p1 * n[0] + p2 * n[1] + p3 * n[2]
    t = (np.float32(0) - s) / (n[0] * n[0] + n[1] * n[1] + n[2] * n[2])
    CP = np.stack([p1 + t * n[0], p2 + t * n[1], p3 + t * n[2]])
    X = lu_solve_f32(np.asarray(R32, dtype=np.float32).reshape(3, 3, order="F"), CP)
    good = (np.abs(X[0].astype(np.float64)) <= n1 / 2) & (np.abs(X[1].astype(np.float64)) <= n2 / 2)
    G = Dind[good]
    return G, D[G], X[0, good], X[1, good]


def centro(FS, n1, n_k1, n2):
    """CentroSymmetricity.m:2-72, literally (flips and permutes)."""
    FS = np.asarray(FS).reshape(-1, order="F")
    M = np.zeros((n1, n2, n1), dtype=np.complex128)

    def flips(a):
        a = a[:, ::-1, :]          # fliplr
        a = a[:, :, ::-1]          # permute(flipud(permute(a,[3 1 2])),[2 3 1])
        return a[::-1, :, :]       # flipud
    if n2 % 2 == 1:
        if n1 % 2 == 1:
            half = FS.reshape(n_k1 + 1, n2, n1, order="F")
            M[:n_k1 + 1] = half
            M[n_k1 + 1:] = np.conj(flips(half[:-1]))
        else:
            ext = FS.reshape(n_k1 + 1, n2, n1 + 1, order="F")
            M[:n_k1 + 1] = ext[:, :, :-1]
            M[n_k1 + 1:] = np.conj(flips(ext[1:-1])[:, :, :-1])
    else:
        if n1 % 2 == 1:
            ext = FS.reshape(n_k1 + 1, n2 + 1, n1, order="F")
            M[:n_k1 + 1] = ext[:, :-1, :]
            M[n_k1 + 1:] = np.conj(flips(ext[:-1])[:, :-1, :])
        else:
            ext = FS.reshape(n_k1 + 1, n2 + 1, n1 + 1, order="F")
            M[:n_k1 + 1] = ext[:, :-1, :-1]
            M[n_k1 + 1:] = np.conj(flips(ext[1:-1])[:, :-1, :-1])
    return M


def hermitian_symmetrize(a):
    """hermitianSymmetrize.m:22-65, literally."""
    d = a.shape
    e = tuple(x + (x % 2 == 0) for x in d)
    inp = np.zeros(e, dtype=np.complex128)
    inp[:d[0], :d[1], :d[2]] = a
    out = inp + np.conj(inp[::-1, ::-1, ::-1])
    nv = (inp != 0).astype(np.float64)
    nv = nv + nv[::-1, ::-1, ::-1]
    nz = nv != 0
    out[nz] = out[nz] / nv[nz]
    return out[:d[0], :d[1], :d[2]]


def make_kspace_indices(shape):
    """make_Kspace_indices.m:16-62."""
    vecs = []
    for n in shape:
        if n % 2 == 0:
            r = n // 2
            vecs.append(np.arange(-r, r) / r)
        elif n == 1:
            vecs.append(np.zeros(1))
        else:
            r = (n - 1) // 2
            vecs.append(np.arange(-r, r + 1) / r)
    Ky, Kx, Kz = np.meshgrid(vecs[0], vecs[1], vecs[2], indexing="ij")
    return np.sqrt(Kx ** 2 + Ky ** 2 + Kz ** 2)


def crop_range(big, ori):
    """1-based [start, end] (My_volumn_index.m:11-28)."""
    if big % 2 == 0:
        s = 1 + (big - ori) // 2 if ori % 2 == 0 else 1 + (big - ori + 1) // 2
    else:
        s = 1 + (big - ori - 1) // 2 if ori % 2 == 0 else 1 + (big - ori) // 2
    return s, s + ori - 1


def paddzero(vol, size):
    out = np.zeros(size, dtype=np.float64)
    sl = tuple(slice(crop_range(b, o)[0] - 1, crop_range(b, o)[1]) for b, o in zip(size, vol.shape))
    out[sl] = vol
    return out


def stripzero(pad, size):
    sl = tuple(slice(crop_range(b, o)[0] - 1, crop_range(b, o)[1]) for b, o in zip(pad.shape, size))
    return pad[sl].copy()


def delay_indicators(mode):
    if mode == 1:
        return np.concatenate([0.95 - 0.1 * np.arange(12), [-10, -10, -10], -0.15 + 0.1 * np.arange(12)])
    if mode == 2:
        return np.concatenate([0.95 - 0.1 * np.arange(12), [-10, -10]])
    return np.full(5, -999.0)


def rfree_candidates(M, nbins, shell):
    """reconstruct.m:47-50: find(M ~= 0 & Q >= edge(s) + resRange & Q < edge(s+1)),
    edge = linspace(0, 1, nbins + 1), resRange = -0.05; 0-based, column-major."""
    Q = make_kspace_indices(M.shape).ravel(order="F")
    lo = shell / nbins + -0.05
    hi = (shell + 1) / nbins
    return np.flatnonzero((M.ravel(order="F") != 0) & (Q >= lo) & (Q < hi)).astype(np.int64)


def reconstruct(M, n_iter, support, mode=3, positivity=True, use_support=True, initial=None, mask=None,
                rfree=None):
    """reconstruct.m:28-194 without the R-factor monitor, with numpy FFTs.  With
    rfree (a list of withheld 0-based centred linear index arrays, already
    cleared in mask) also returns Rfree (shells x iterations, :137-146)."""
    n = M.shape
    D = support.shape
    S = np.fft.ifftshift(paddzero(support.astype(np.float64), n))
    x = np.fft.ifftshift(paddzero(initial if initial is not None else np.zeros(D), n))
    Q = make_kspace_indices(n)
    if mask is None:
        mask = M != 0
    Emask = (M != 0) & mask
    ci = np.zeros(n)
    ci[Emask] = 1 - Q[Emask]
    delay = delay_indicators(mode)
    m = len(delay)
    changes = mround(1 + np.arange(m) * (n_iter - 1) / (m - 1)).astype(int) if m > 1 else np.array([n_iter])
    Ms = np.fft.ifftshift(M)
    Es = np.fft.ifftshift(Emask)
    cis = np.fft.ifftshift(ci)
    denom = np.abs(M[Emask]).sum()
    best_err = 1e30
    best = None
    cur = 0
    Cs = None
    errK = np.zeros(n_iter)
    Rf = np.zeros((len(rfree) if rfree is not None else 0, n_iter))
    for it in range(1, n_iter + 1):
        if cur < m and it == changes[cur]:
            last = np.nonzero(changes == it)[0][-1]
            Cs = (cis > delay[last]) & Es
            cur = last + 1
            best_err = 1e30
        if positivity:
            x[x < 0] = 0
        if use_support:
            x = x * S
        k = np.fft.fftn(x)
        errK[it - 1] = np.abs(np.abs(k[Es]) - np.abs(Ms[Es])).sum() / denom
        if rfree is not None:
            kc = np.fft.fftshift(k).ravel(order="F")
            Mf = M.ravel(order="F")
            for sh, idx in enumerate(rfree):
                Rf[sh, it - 1] = np.abs(kc[idx] - Mf[idx]).sum() / np.abs(Mf[idx]).sum()
        if errK[it - 1] < best_err:
            best_err = errK[it - 1]
            best = x.copy()
        k[Cs] = Ms[Cs]
        x = np.real(np.fft.ifftn(k))
    if rfree is not None:
        return stripzero(np.fft.fftshift(best), D), errK, Rf
    return stripzero(np.fft.fftshift(best), D), errK


def project(vol, R):
    """Trilinear projector, sum over dim 3 of Vol(R*[X;Y;Z]) with 0 outside."""
    n1, n2, n3 = vol.shape
    X, Y, Z = np.meshgrid(np.arange(n1) - n1 // 2, np.arange(n2) - n2 // 2, np.arange(n3) - n3 // 2,
                          indexing="ij")
    pos = np.stack([X.ravel(), Y.ravel(), Z.ravel()]).astype(np.float64)
    r = R @ pos
    x = r[0] + n1 // 2
    y = r[1] + n2 // 2
    z = r[2] + n3 // 2
    inside = (x >= 0) & (y >= 0) & (z >= 0) & (x <= n1 - 1) & (y <= n2 - 1) & (z <= n3 - 1)
    i = np.clip(np.floor(x).astype(int), 0, n1 - 2)
    j = np.clip(np.floor(y).astype(int), 0, n2 - 2)
    k = np.clip(np.floor(z).astype(int), 0, n3 - 2)
    fx, fy, fz = x - i, y - j, z - k
    i, j, k = (np.where(inside, a, 0) for a in (i, j, k))
    V = vol

    def g(a, b, c):
        return V[a, b, c]
    c00 = g(i, j, k) * (1 - fx) + g(i + 1, j, k) * fx
    c10 = g(i, j + 1, k) * (1 - fx) + g(i + 1, j + 1, k) * fx
    c01 = g(i, j, k + 1) * (1 - fx) + g(i + 1, j, k + 1) * fx
    c11 = g(i, j + 1, k + 1) * (1 - fx) + g(i + 1, j + 1, k + 1) * fx
    c0 = c00 * (1 - fy) + c10 * fy
    c1 = c01 * (1 - fy) + c11 * fy
    val = np.where(inside, c0 * (1 - fz) + c1 * fz, 0.0)
    return val.reshape(n1, n2, n3).sum(axis=2)


def _sincosd(x):
    """sind/cosd exact at multiples of 90 degrees (MATLAB's sind/cosd)."""
    r = np.remainder(x + 180.0, 360.0) - 180.0
    q = np.round(r / 90.0)
    t = np.deg2rad(r - 90.0 * q)
    s, c = np.sin(t), np.cos(t)
    qi = int(q) % 4
    return [(s, c), (c, -s), (-s, -c), (-c, s)][qi]


def fill_in_fourier_grid(projs, angles, ratio, cutoff, allow_multiple=True):
    """fillInFourierGrid.m:27-168 statement by statement (FP64 values, FP32
    coordinates and weights, accumarray as an ordered np.add.at)."""
    D1, D2, P = projs.shape
    m = D2 * ratio if D2 % 2 == 0 else 1 + (D2 - 1) * ratio
    m = int(round(m))
    nc = np.float32(mround((m + 1) / 2))
    a = (np.arange(1, m + 1) - nc).astype(np.float32)
    ky, kx = np.meshgrid(a, a)            # kx along dim 1, ky along dim 2
    kx = kx.reshape(-1, order="F")
    ky = ky.reshape(-1, order="F")
    kz = np.zeros_like(kx)
    kM = np.zeros((m, m, P), dtype=np.complex128)
    for p in range(P):
        pad = paddzero(projs[:, :, p], (m, m))
        kM[:, :, p] = np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(pad)))
    mX = np.zeros((m * m, P), dtype=np.float32)
    mY = np.zeros_like(mX)
    mZ = np.zeros_like(mX)
    for p in range(P):
        sf, cf = _sincosd(angles[p, 0])
        st, ct = _sincosd(angles[p, 1])
        sp, cp = _sincosd(angles[p, 2])
        R = np.array([[cp * ct * cf - sp * sf, cp * ct * sf + sp * cf, -cp * st],
                      [-sp * ct * cf - cp * sf, -sp * ct * sf + cp * cf, sp * st],
                      [st * cf, st * sf, ct]])
        Rt = R.T.astype(np.float32)
        mX[:, p] = Rt[0, 0] * kx + Rt[0, 1] * ky + Rt[0, 2] * kz
        mY[:, p] = Rt[1, 0] * kx + Rt[1, 1] * ky + Rt[1, 2] * kz
        mZ[:, p] = Rt[2, 0] * kx + Rt[2, 1] * ky + Rt[2, 2] * kz
    mX = mX.reshape(-1, order="F"); mY = mY.reshape(-1, order="F"); mZ = mZ.reshape(-1, order="F")
    kv = kM.reshape(-1, order="F")
    good = kv != -999
    mX, mY, mZ, kv = mX[good], mY[good], mZ[good], kv[good]
    s = int(mround(cutoff)) if allow_multiple else 0
    inds, vals, dists = [], [], []
    for ys in range(-s, s + 1):
        for xs in range(-s, s + 1):
            for zs in range(-s, s + 1):
                tX = (np.sign(mX) * np.floor(np.abs(mX) + np.float32(0.5))).astype(np.float32) + np.float32(xs)
                tY = (np.sign(mY) * np.floor(np.abs(mY) + np.float32(0.5))).astype(np.float32) + np.float32(ys)
                tZ = (np.sign(mZ) * np.floor(np.abs(mZ) + np.float32(0.5))).astype(np.float32) + np.float32(zs)
                dx, dy, dz = mX - tX, mY - tY, mZ - tZ
                d = np.sqrt(dx * dx + dy * dy + dz * dz).astype(np.float32)
                tY1, tZ1, tX1 = tY + nc, tZ + nc, tX + nc
                ok = ~((tX1 > m) | (tX1 < 1) | (tY1 > m) | (tY1 < 1) | (tZ1 > m) | (tZ1 < 1)) & (d.astype(np.float64) <= cutoff)
                ix = tX1[ok].astype(np.int64) - 1
                iy = tY1[ok].astype(np.int64) - 1
                iz = tZ1[ok].astype(np.int64) - 1
                inds.append(ix + m * (iy + m * iz))
                vals.append(kv[ok])
                dists.append(d[ok])
    ind = np.concatenate(inds)
    val = np.concatenate(vals)
    w = np.float32(1.0) / (np.concatenate(dists) + np.float32(1e-5))
    num = np.zeros(m ** 3, dtype=np.complex128)
    ws = np.zeros(m ** 3, dtype=np.float64)
    np.add.at(num, ind, val * w.astype(np.float64))
    np.add.at(ws, ind, w.astype(np.float64))
    pos = ws > 0
    num[pos] = num[pos] / ws[pos]
    K = hermitian_symmetrize(num.reshape((m, m, m), order="F"))
    rec = stripzero(np.real(np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(K)))), (D1, D2, D1))
    return K, rec, ind.size


def _keys_dense(x, n):
    """Dense length-n weights of Keys' cubic convolution (a = -1/2) at x, with
    the boundary samples f(-1) = 3f(0) - 3f(1) + f(2) and f(n) = 3f(n-1) -
    3f(n-2) + f(n-3) folded in; None outside [0, n-1]."""
    if not (0 <= x <= n - 1):
        return None
    i = min(max(int(np.floor(x)), 0), n - 2)
    w = np.zeros(n)
    for a in range(i - 1, i + 3):
        s = abs(x - a)
        k = 1.5 * s ** 3 - 2.5 * s ** 2 + 1 if s <= 1 else (-0.5 * s ** 3 + 2.5 * s ** 2 - 4 * s + 2 if s < 2 else 0.0)
        if a < 0:
            w[0] += 3 * k; w[1] -= 3 * k; w[2] += k
        elif a > n - 1:
            w[n - 1] += 3 * k; w[n - 2] -= 3 * k; w[n - 3] += k
        else:
            w[a] += k
    return w


def project_cubic(vol, R):
    """calculate3Dprojection_RealSpaceinterp with interp3 'cubic' read as Keys
    cubic convolution: each rotated sample as a tensor product of dense 1-D
    weight vectors."""
    n1, n2, n3 = vol.shape
    c = (n1 // 2, n2 // 2, n3 // 2)
    out = np.zeros((n1, n2))
    for i in range(n1):
        for j in range(n2):
            s = 0.0
            for k in range(n3):
                X = np.array([i - c[0], j - c[1], k - c[2]], dtype=np.float64)
                r = R @ X + np.array(c)
                w1, w2, w3 = _keys_dense(r[0], n1), _keys_dense(r[1], n2), _keys_dense(r[2], n3)
                if w1 is None or w2 is None or w3 is None:
                    continue
                s += np.einsum("a,b,c,abc->", w1, w2, w3, vol)
            out[i, j] = s
    return out
