"""An independent restatement, in plain Python (IEEE f64 floats, correctly
rounded math.sqrt, no fused operations), of the reference's SVD
(src/math/svd.rs: computeSVD = factorize + factorize_hh, unpack, diagonalize
+ chop + qrstep / qrstep_middle / qrstep_end / qrstep_eigenvalue /
qrstep_cols2 + computeGivens / computeSchur, singularize; SVD::solve =
thresholds + solveSVD), operation for operation in the reference's order,
checked bit for bit against the oracle's SVD, which DualContouring's and
ExtendedMarchingCubes' feature placement (on the GPU too) follow; and of the
feature placers built on it (feature/mod.rs TangentPlanes, feature/qef.rs
MinimiseQEF, feature/particle_minimisation.rs) in numpy float32."""
import math

import numpy as np
import pytest

import oracle


def factorize_hh(m, ptrs):
    """Householder vector of the elements m[r][c] for (r, c) in ptrs."""
    n = len(ptrs)
    get = lambda k: m[ptrs[k][0]][ptrs[k][1]]

    def put(k, val):
        m[ptrs[k][0]][ptrs[k][1]] = val

    tau = 0.0
    if n > 1:
        if n == 2:
            xnorm = abs(get(1))
        else:
            scl, ssq = 0.0, 1.0
            for i in range(1, n):
                x = abs(get(i))
                if x != 0.0:
                    if scl < x:
                        ssq = 1.0 + ssq * (scl / x) * (scl / x)
                        scl = x
                    else:
                        ssq += x / scl * (x / scl)
            xnorm = scl * math.sqrt(ssq)
        if xnorm != 0.0:
            alpha = get(0)
            beta = math.sqrt(alpha * alpha + xnorm * xnorm)
            if alpha >= 0.0:
                beta = -beta
            tau = (beta - alpha) / beta
            scl = 1.0 / (alpha - beta)
            put(0, beta)
            for i in range(1, n):
                put(i, get(i) * scl)
    return tau


def factorize(mat, tau_u, tau_v, rows):
    for i in range(3):
        ptrs = [(q + i, i) for q in range(rows - i)]
        tau = factorize_hh(mat, ptrs)
        tau_u[i] = tau
        if i + 1 < 3:
            if tau != 0.0:
                for x in range(i + 1, 3):
                    wx = mat[i][x]
                    for y in range(i + 1, rows):
                        wx += mat[y][x] * mat[ptrs[y - i][0]][ptrs[y - i][1]]
                    tau_wx = tau * wx
                    mat[i][x] -= tau_wx
                    for y in range(i + 1, rows):
                        mat[y][x] -= tau_wx * mat[ptrs[y - i][0]][ptrs[y - i][1]]
            rp = [(i, i + 1), (i, i + 2)] if i == 0 else [(i, i + 1)]
            tau = factorize_hh(mat, rp)
            tau_v[i] = tau
            if tau != 0.0:
                for y in range(i + 1, rows):
                    wy = mat[y][i + 1]
                    if i == 0:
                        wy += mat[y][i + 2] * mat[rp[1][0]][rp[1][1]]
                    tau_wy = tau * wy
                    mat[y][i + 1] -= tau_wy
                    if i == 0:
                        mat[y][i + 2] -= tau_wy * mat[rp[1][0]][rp[1][1]]


def unpack(u, v, tau_u, tau_v, rows):
    for r in range(3):
        for c in range(3):
            v[r][c] = 1.0 if r == c else 0.0
    for i in (1, 0):
        tau = tau_v[i]
        if tau != 0.0:
            for x in range(i + 1, 3):
                wx = v[i + 1][x]
                for y in range(i + 2, 3):
                    wx += v[y][x] * u[i][y]
                tau_wx = tau * wx
                v[i + 1][x] -= tau_wx
                for y in range(i + 2, 3):
                    v[y][x] -= tau_wx * u[i][y]
    for i in range(2):
        tau_v[i] = u[i][i + 1]
    for i in (2, 1, 0):
        tau = tau_u[i]
        tau_u[i] = u[i][i]
        if tau == 0.0:
            u[i][i] = 1.0
            if i < 2:
                u[i][2] = 0.0
                if i < 1:
                    u[i][1] = 0.0
            for y in range(i + 1, rows):
                u[y][i] = 0.0
        else:
            for x in range(i + 1, 3):
                wx = 0.0
                for y in range(i + 1, rows):
                    wx += u[y][x] * u[y][i]
                tau_wx = tau * wx
                u[i][x] = -tau_wx
                for y in range(i + 1, rows):
                    u[y][x] -= tau_wx * u[y][i]
            for y in range(i + 1, rows):
                u[y][i] = u[y][i] * -tau
            u[i][i] = 1.0 - tau


def givens(a, b):
    if b == 0.0:
        return 1.0, 0.0
    if abs(b) > abs(a):
        t = -a / b
        s1 = 1.0 / math.sqrt(1.0 + t * t)
        return s1 * t, s1
    t = -b / a
    c1 = 1.0 / math.sqrt(1.0 + t * t)
    return c1, c1 * t


def schur(a1, a2, a3):
    apq = a1 * a2 * 2.0
    if apq == 0.0:
        return 1.0, 0.0
    tau = (a2 * a2 + (a3 + a1) * (a3 - a1)) / apq
    if tau >= 0.0:
        t = 1.0 / (tau + math.sqrt(1.0 + tau * tau))
    else:
        t = -1.0 / (math.sqrt(1.0 + tau * tau) - tau)
    c = 1.0 / math.sqrt(1.0 + t * t)
    return c, t * c


def rot(m, nrows, p, q, c, s):
    for i in range(nrows):
        ip, iq = m[i][p], m[i][q]
        m[i][p] = ip * c - iq * s
        m[i][q] = ip * s + iq * c


def qrstep_middle(u, tu, tv, rows, cols, col):
    x, y = tv[col], tu[col + 1]
    for j in range(col, cols - 1):
        c, s = givens(y, -x)
        for i in range(rows):  # the reference rotates column `col` with j + 1
            uip, uiq = u[i][col], u[i][j + 1]
            u[i][col] = uip * c - uiq * s
            u[i][j + 1] = uip * s + uiq * c
        tu[j + 1] = x * s + y * c
        if j == col:
            tv[j] = x * c - y * s
        if j < cols - 2:
            z = tv[j + 1]
            tv[j + 1] *= c
            x = z * -s
            y = tu[j + 2]


def qrstep_end(v, tu, tv):
    x, y = tu[1], tv[1]
    for k in (1, 0):
        c, s = givens(x, y)
        for i in range(3):
            vip, viq = v[i][k], v[i][2]
            v[i][k] = vip * c - viq * s
            v[i][2] = vip * s + viq * c
        tu[k] = x * c - y * s
        if k == 1:
            tv[k] = x * s + y * c
        if k > 0:
            z = tv[k - 1]
            tv[k - 1] *= c
            x = tu[k - 1]
            y = z * s


def qrstep_eigenvalue(tu, tv):
    ta = tu[1] * tu[1] + tv[0] * tv[0]
    tb = tu[2] * tu[2] + tv[1] * tv[1]
    tab = tu[1] * tv[1]
    dt = (ta - tb) / 2.0
    if dt >= 0.0:
        return tb - tab * tab / (dt + math.sqrt(dt * dt + tab * tab))
    return tb + tab * tab / (math.sqrt(dt * dt + tab * tab) - dt)


def qrstep_cols2(u, v, tu, tv, rows):
    if tu[0] == 0.0:
        c, s = givens(tv[0], tu[1])
        tu[0] = tv[0] * c - tu[1] * s
        tv[0] = tv[0] * s + tu[1] * c
        tu[1] = 0.0
        rot(u, rows, 0, 1, c, s)
        for i in range(3):
            v[i][0], v[i][1] = v[i][1], v[i][0]
    elif tu[1] == 0.0:
        c, s = givens(tu[0], tv[0])
        tu[0] = tu[0] * c - tv[0] * s
        tv[0] = 0.0
        rot(v, 3, 0, 1, c, s)
    else:
        c, s = schur(tu[0], tv[0], tu[1])
        a11 = tu[0] * c - tv[0] * s
        a21 = -tu[1] * s
        a12 = tu[0] * s + tv[0] * c
        a22 = tu[1] * c
        rot(v, 3, 0, 1, c, s)
        if a11 * a11 + a21 * a21 < a12 * a12 + a22 * a22:
            a11, a12 = a12, a11
            a21, a22 = a22, a21
            for i in range(3):
                v[i][0], v[i][1] = v[i][1], v[i][0]
        c, s = givens(a11, a21)
        tu[0] = a11 * c - a21 * s
        tv[0] = a12 * c - a22 * s
        tu[1] = a12 * s + a22 * c
        rot(u, rows, 0, 1, c, s)


def qrstep(u, v, tu, tv, rows, cols):
    if cols == 2:
        qrstep_cols2(u, v, tu, tv, rows)
        return
    assert cols != 1  # the reference writes through a null pointer there
    for i in range(cols - 1):
        if tu[i] == 0.0:
            qrstep_middle(u, tu, tv, rows, cols, i)
            return
    if tu[cols - 1] == 0.0:
        qrstep_end(v, tu, tv)
        return
    mu = qrstep_eigenvalue(tu, tv)
    y = tu[0] * tu[0] - mu
    z = tu[0] * tv[0]
    ak = bk = 0.0
    zk = 0.0
    ap, bp, aq = tu[0], tv[0], tu[1]
    for k in range(cols - 1):
        c, s = givens(y, z)
        rot(v, 3, k, k + 1, c, s)
        bk1 = bk * c - z * s
        ap1 = ap * c - bp * s
        bp1 = ap * s + bp * c
        zp1 = aq * -s
        aq1 = aq * c
        if k > 0:
            tv[k - 1] = bk1
        ak, bk, zk, ap = ap1, bp1, zp1, aq1
        bp = tv[k + 1] if k < cols - 2 else 0.0
        y, z = ak, zk
        c, s = givens(y, z)
        rot(u, rows, k, k + 1, c, s)
        ak1 = ak * c - zk * s
        bk1 = bk * c - ap * s
        zk1 = bp * -s
        ap1 = bk * s + ap * c
        bp1 = bp * c
        tu[k] = ak1
        ak, bk, zk, ap, bp = ak1, bk1, zk1, ap1, bp1
        aq = tu[k + 2] if k < cols - 2 else 0.0
        y, z = bk, zk
    tv[cols - 2] = bk
    tu[cols - 1] = ap


def chop(a, b, n):
    ai = a[0]
    for i in range(n - 1):
        bi, ai1 = b[i], a[i + 1]
        if abs(bi) < 1e-5 * (abs(ai) + abs(ai1)):
            b[i] = 0.0
        ai = ai1


def diagonalize(u, v, tu, tv, rows):
    chop(tu, tv, 3)
    b = 2
    while b > 0:
        if tv[b - 1] == 0.0:
            b -= 1
        else:
            a = b - 1
            while a > 0 and tv[a - 1] != 0.0:
                a -= 1
            n = b - a + 1
            u1 = [[0.0] * 3 for _ in range(12)]
            v1 = [[0.0] * 3 for _ in range(3)]
            for j in range(a, b + 1):
                for i in range(rows):
                    u1[i][j - a] = u[i][j]
                for i in range(3):
                    v1[i][j - a] = v[i][j]
            sub_u, sub_v = tu[a:], tv[a:]
            qrstep(u1, v1, sub_u, sub_v, rows, n)
            tu[a:], tv[a:] = sub_u, sub_v
            for j in range(a, b + 1):
                for i in range(rows):
                    u[i][j] = u1[i][j - a]
                for i in range(3):
                    v[i][j] = v1[i][j - a]
            sub_u, sub_v = tu[a:], tv[a:]
            chop(sub_u, sub_v, n)
            tu[a:], tv[a:] = sub_u, sub_v


def singularize(u, v, d, rows):
    for j in range(3):
        if d[j] < 0.0:
            for i in range(3):
                v[i][j] = -v[i][j]
            d[j] = -d[j]
    for i in range(3):
        d_max, i_max = d[i], i
        for j in range(i + 1, 3):
            if d[j] > d_max:
                d_max, i_max = d[j], j
        if i_max != i:
            d[i], d[i_max] = d[i_max], d[i]
            for y in range(rows):
                u[y][i], u[y][i_max] = u[y][i_max], u[y][i]
            for y in range(3):
                v[y][i], v[y][i_max] = v[y][i_max], v[y][i]


def compute_svd(mat):
    rows = len(mat)
    u = [[0.0] * 3 for _ in range(12)]
    for i in range(rows):
        u[i] = [float(x) for x in mat[i]]
    v = [[0.0] * 3 for _ in range(3)]
    d = [0.0, 0.0, 0.0]  # tau_u aliases d
    tau_v = [0.0, 0.0]
    factorize(u, d, tau_v, rows)
    unpack(u, v, d, tau_v, rows)
    diagonalize(u, v, d, tau_v, rows)
    singularize(u, v, d, rows)
    return u, v, d


def solve(u, v, d, b, rows):
    d = list(d)
    for k in (2, 1, 0):
        if d[k] < 0.1:
            d[k] = 0.0
    w = [0.0, 0.0, 0.0]
    for i in range(rows):
        if b[i] != 0.0:
            for j in range(3):
                w[j] += b[i] * u[i][j]
    for i in range(3):
        if d[i] != 0.0:
            w[i] /= d[i]
    x = []
    for i in range(3):
        tmp = 0.0
        for j in range(3):
            tmp += w[j] * v[i][j]
        x.append(tmp)
    return x


def _systems():
    rng = np.random.default_rng(17)
    out = []
    for rows in range(3, 13):
        for _ in range(12):
            a = rng.normal(size=(rows, 3))
            a /= np.linalg.norm(a, axis=1, keepdims=True)
            out.append((a, rng.normal(size=rows) * 0.05))
    # structured: axis-aligned normals (cube corners and edges), repeated rows, a zero row
    axes = np.eye(3)
    out.append((np.array([axes[0]] * 4 + [axes[1]] * 4), np.linspace(-0.01, 0.01, 8)))
    out.append((np.array([axes[0], axes[1], axes[2], axes[0], axes[1], axes[2], axes[0], axes[1]]), np.arange(8) * 0.01))
    out.append((np.array([[0.6, 0.8, 0.0]] * 6 + [[0.0, 0.0, 0.0]] * 2), np.full(8, 0.02)))
    out.append((np.array([[0.0, 0.0, 1.0]] * 3), np.zeros(3)))
    # a normal component that is zero in every plane (axis-aligned surfaces, a
    # cylinder's side): exact zeros on the bidiagonal reach qrstep_middle and
    # qrstep_end
    for rows in range(3, 13):
        for col in range(3):
            a = rng.normal(size=(rows, 3))
            a[:, col] = 0.0
            a /= np.linalg.norm(a, axis=1, keepdims=True)
            out.append((a, rng.normal(size=rows) * 0.05))
    # small integer rows with two equal columns: an exact zero last on the
    # diagonal under a non-zero superdiagonal reaches qrstep_end
    irng = np.random.default_rng(3)
    for rows in range(3, 9):
        for _ in range(6):
            a = irng.integers(-2, 3, size=(rows, 3)).astype(np.float64)
            a[:, 1] = a[:, 0]
            out.append((a, irng.normal(size=rows) * 0.05))
    return out


SYSTEMS = _systems()


@pytest.mark.parametrize("k", range(len(SYSTEMS)))
def test_independent_svd_matches_oracle(k):
    """Singular values and the truncated solution, bit for bit."""
    a, b = SYSTEMS[k]
    u, v, d = compute_svd(a.tolist())
    x = solve(u, v, d, b.tolist(), len(a))
    od, ox = oracle.svd_solve(a, b)
    assert np.array_equal(np.array(d), od), (d, od)
    assert np.array_equal(np.array(x), ox), (x, ox)


# -- feature placement (DualContouring's corners) --------------------------------
F = np.float32
FEATURE_ANGLE = F(0.8660254037844387)


def _dot(a, b):  # (a * b).component_sum() == (x + y) + z
    p = a * b
    return F(F(p[0] + p[1]) + p[2])


def _cross(a, r):
    return np.array([a[1] * r[2] - a[2] * r[1], a[2] * r[0] - a[0] * r[2], a[0] * r[1] - a[1] * r[0]], F)


def _normalised_or_zero(v):
    ln = np.sqrt(F(F(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))
    return np.zeros(3, F) if abs(ln) < F(1.1920929e-07) else v / ln


def tangent_planes(vertices, normals):
    """TangentPlanes::new (feature/mod.rs:91-148): (normals, d, centre of mass, topology)."""
    com = np.zeros(3, F)
    axis = np.zeros(3, F)
    min_angle = F(3.40282347e38)
    count = F(0.0)
    for i in range(len(vertices)):
        for j in range(len(vertices)):
            angle = _dot(normals[i], normals[j])
            if angle < min_angle:
                axis = _cross(normals[i], normals[j])
                min_angle = angle
        com = com + vertices[i]
        count = F(count + F(1.0))
    com = com / count
    if min_angle > FEATURE_ANGLE:
        topo = 0
    else:
        axis = _normalised_or_zero(axis)
        min_c, max_c = F(1.0), F(-1.0)
        for n in normals:
            c = _dot(axis, n)
            min_c, max_c = np.fmin(min_c, c), np.fmax(max_c, c)
        c = np.fmax(abs(min_c), abs(max_c))
        c = np.sqrt(F(F(1.0) - c * c))
        topo = 1 if c > FEATURE_ANGLE else 2
    d = [_dot(vertices[i] - com, normals[i]) for i in range(len(vertices))]
    return normals, d, com, topo


def minimise_qef(vertices, normals):
    """MinimiseQEF::place_feature_with_tangents (feature/qef.rs:36-68)."""
    nrm, d, com, topo = tangent_planes(vertices, normals)
    if topo == 0:
        return com
    u, v, s = compute_svd([[float(x) for x in n] for n in nrm])
    if topo == 1:  # an edge: zero the smallest singular value
        s_min, idx = 1.7976931348623157e308, 0
        for i in range(3):
            if s[i] < s_min:
                s_min, idx = s[i], i
        s[idx] = 0.0
    x = solve(u, v, s, [float(di) for di in d], len(nrm))
    return com + np.array([F(x[0]), F(x[1]), F(x[2])], F)


def particle_placement(corners, normals):
    """ParticleBasedMinimisation::place_feature_in_cell (particle_minimisation.rs:27-72)."""
    nrm, d, com, _ = tangent_planes(corners, normals)
    mfs = F(corners[6][0] - corners[0][0])
    particle = com
    forces = [np.zeros(3, F) for _ in range(8)]
    for i in range(8):
        for j in range(8):
            dist = F(_dot(nrm[j], corners[i]) - d[j])  # Plane::distance
            closest = corners[i] - nrm[j] * dist  # point_closest_to
            forces[i] = forces[i] + (corners[i] - closest)
    span = np.array([corners[1][0], corners[3][1], corners[4][2]], F) - corners[0]
    for _ in range(100):
        f = (particle - corners[0]) / span
        lx = lambda a, b: F(F(1.0) - f[0]) * a + f[0] * b
        c00, c01 = lx(forces[0], forces[1]), lx(forces[4], forces[5])
        c10, c11 = lx(forces[3], forces[2]), lx(forces[7], forces[6])
        c0 = F(F(1.0) - f[1]) * c00 + f[1] * c10
        c1 = F(F(1.0) - f[1]) * c01 + f[1] * c11
        force = (F(F(1.0) - f[2]) * c0 + f[2] * c1) * F(0.05) * mfs
        particle = particle + force
        if F(F(force[0] * force[0] + force[1] * force[1]) + force[2] * force[2]) < F(F(0.02) * mfs):
            break
    return particle


def _cells():
    """Active cells of the CSG scene at new(9) (corners and normalised normals),
    and synthetic cells whose normals form creases and corners."""
    from isosurface_gb300 import scenes
    from isosurface_gb300 import source as S
    prog = oracle.Program(S.lower(scenes.csg()))
    n = 9
    inv = F(1.0) / F(n - 1)
    out = []
    offs = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    for z in range(n):
        for y in range(n - 1):
            for x in range(n - 1):
                corners = np.array([(x + a, y + b, z + c) for a, b, c in offs], F) * inv
                vals = prog.sample_scalar(corners)
                cube = sum(1 << i for i in range(8) if not vals[i] > F(0.0))
                if cube in (0, 255):
                    continue
                normals = np.array([_normalised_or_zero(nm) for nm in prog.sample_normal(corners)], F)
                out.append((corners, normals))
    rng = np.random.default_rng(9)
    axes = np.eye(3, dtype=F)
    for k in range(40):
        corners = (np.array(offs, F) * F(0.125) + F(rng.uniform(0, 0.8))).astype(F)
        pick = [axes[0], axes[1]] if k % 2 else [axes[0], axes[1], axes[2]]
        normals = np.array([pick[i % len(pick)] for i in range(8)], F)
        normals = np.array([_normalised_or_zero(nm + F(0.01) * rng.normal(size=3).astype(F)) for nm in normals], F)
        out.append((corners, normals))
    return out


CELLS = _cells()


@pytest.mark.parametrize("placer", [0, 1])
def test_independent_feature_placement_matches_oracle(placer):
    topologies = set()
    for corners, normals in CELLS:
        want, topo = oracle.place_feature(corners, normals, placer)
        got = minimise_qef(corners, normals) if placer == 0 else particle_placement(corners, normals)
        assert np.array_equal(got, want), (placer, corners[0], got, want)
        topologies.add(topo)
    assert topologies == {0, 1, 2}
