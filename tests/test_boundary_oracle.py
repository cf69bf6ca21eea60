"""The step-boundary oracle (rock properties, displacement-limited time step) against direct
numpy transcriptions of the reference's formulas."""
import numpy as np
import pytest

from boundary_cases import porosity_fields, rock_golden_markers, rock_tables, sediment


@pytest.fixture(scope="module")
def B():
    from oracle import boundary
    boundary.build()
    return boundary


def markers(eb, M=3000, seed=5):
    rng = np.random.default_rng(seed)
    g = eb.synthetic.staggered_grid(np.linspace(0, 100e3, 11), np.linspace(0, 150e3, 16))
    mk = {"x": rng.uniform(-1e3, 101e3, M), "y": rng.uniform(0, 150e3, M), "matid": rng.integers(1, 5, M).astype(np.int16),
          "pr": rng.uniform(1e5, 4e9, M), "tk": rng.uniform(273.0, 1700.0, M), "inside": np.where(rng.random(M) < 0.95, 1, -1).astype(np.int8)}
    for k in ("rho", "rhocp", "kt", "ha"):
        mk[k] = rng.uniform(0, 1, M)
    mk.update(porosity_fields(M))
    return g, mk


def numpy_props(mk, mat_rho, mat_cp, mat_kt, dm, cm, km, Ttop, cpmax, sed=None):
    id_ = mk["matid"].astype(np.int64) - 1
    rs, a, b = mat_rho[id_, 0], mat_rho[id_, 1], mat_rho[id_, 2]
    T, P, y = mk["tk"], mk["pr"], mk["y"]
    rho = [rs * (1.0 - a * (T - 298.15)) * (1.0 + b * (P - 1e5)), rs * (1.0 - a * (T - Ttop)),
           rs * (1.0 - a * (T - 830.0))][dm]
    cp20 = mat_cp[id_]
    tc = T - 273.0
    cpw = np.minimum(cp20 * (0.953 + 2.29e-3 * tc - 2.835e-6 * tc ** 2 + 1.191e-9 * tc ** 3), cpmax)
    rhocp = rho * (cp20 if cm == 0 else cpw)
    k0, ka = mat_kt[id_, 0], mat_kt[id_, 1]
    k = [(k0 + ka / (T + 77.0)) * np.exp(0.00004 * P / 1e6), k0, k0 / (1.0 + ka * (T - Ttop) / Ttop),
         np.where(y > 110000.0, 39.25, k0), np.where(y > 110000.0, 0.1 * 2.25 * 1330.0 / 4.5, k0),
         np.where(k0 <= 20.0, 358.0 * (1.0227 * k0 - 1.882) * (1.0 / T - 0.00068) + 1.84, k0)][km]
    ha = a * T
    if sed is not None:
        ymud = np.interp(mk["x"], sed["topo_x"], sed["topo_y"])
        ysub = np.maximum(y - ymud, mk["max_burial_depth"])
        phi = mk["porosity_initial"] * np.exp(-(1.0 / mk["decay_depth"]) * ysub)
        s = np.isin(mk["matid"], sed["matids"])
        k = np.where(s, k * (1 - phi) + sed["conductivity_water"] * phi, k)
        rho = np.where(s, rho * (1 - phi) + sed["density_water"] * phi, rho)
        rhocp = np.where(s, rho * (cp20 * (1 - phi) + sed["heat_capacity_water"] * phi), rhocp)
    ins = mk["inside"] == 1
    return {n: np.where(ins, v, mk[n]) for n, v in (("rho", rho), ("rhocp", rhocp), ("kt", k), ("ha", ha))}


@pytest.mark.parametrize("dm,cm,km", [(d, c, k) for d in range(3) for c in range(2) for k in range(6)])
def test_rock_properties(eb, B, dm, cm, km):
    g, mk = markers(eb)
    tabs = rock_tables(4)
    got = B.rock_properties(mk, *tabs, dm, cm, km, 273.15, 1200.0)
    want = numpy_props(mk, *tabs, dm, cm, km, 273.15, 1200.0)
    for n in want:
        np.testing.assert_allclose(got[n], want[n], rtol=2e-15, atol=0, err_msg=n)


def test_rock_properties_porosity(eb, B):
    g, mk = markers(eb)
    tabs = rock_tables(4)
    sed = sediment(g)
    got = B.rock_properties(mk, *tabs, 0, 1, 0, 273.15, 1200.0, iuse_por=1, sed=sed)
    want = numpy_props(mk, *tabs, 0, 1, 0, 273.15, 1200.0, sed=sed)
    for n in want:
        np.testing.assert_allclose(got[n], want[n], rtol=1e-13, atol=0, err_msg=n)


@pytest.mark.parametrize("local", [0, 1])
def test_timestep_displacement_limit(eb, B, local):
    rng = np.random.default_rng(7)
    x = np.concatenate([[0.0], np.cumsum(rng.uniform(400.0, 1200.0, 30))])
    y = np.concatenate([[0.0], np.cumsum(rng.uniform(300.0, 900.0, 20))])
    g = eb.synthetic.staggered_grid(x, y)
    vx = rng.normal(0, 1e-9, (g.ynum + 1, g.xnum))
    vy = rng.normal(0, 1e-9, (g.ynum, g.xnum + 1))
    vx[3, 4] = 0.0
    dt_old, displ = 1e13, 0.4
    got = B.timestep_displacement_limit(g, vx, vy, displ, local, dt_old)
    if local == 0:
        want = min(dt_old, displ * g.xstpavg / np.abs(vx).max(), displ * g.ystpavg / np.abs(vy).max())
    else:
        xs, ys = g.xstp_b, g.ystp_b
        cx = np.concatenate([[xs[0]], np.minimum(xs[:-1], xs[1:]), [xs[-1]]])
        cy = np.concatenate([[ys[0]], np.minimum(ys[:-1], ys[1:]), [ys[-1]]])
        with np.errstate(divide="ignore"):
            lx = np.where(vx != 0, displ * cx[None, :] / np.abs(vx), np.inf)
            ly = np.where(vy != 0, displ * cy[:, None] / np.abs(vy), np.inf)
        want = min(dt_old, lx.min(), ly.min())
    assert got == want


# Philox-4x32-10 known answers published with the Random123 library (Salmon, Moraes, Dror,
# Shaw, SC 2011): (counter, key) -> output
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_known_answers(B, ctr, key, want):
    assert B.philox4x32_10(ctr, key) == want


def test_recycle_uniforms_library_matches_oracle(eb, B):
    """The product's host copy of the generator (eb_recycle_uniforms, a pure host function)
    gives the oracle's numbers, including 64-bit indices."""
    import ctypes as C
    eb.build()
    from earthbox_gb300 import _abi
    lib = _abi.load()
    for seed, step, stream, j in [(0, 0, 0, 0), (12345, 7, 1, 42), (2**63 + 5, 2**31 - 1, 2, 2**33 + 9),
                                  (99, 3, 0, 10**6)]:
        u0, u1 = C.c_double(), C.c_double()
        lib.eb_recycle_uniforms(seed, step, stream, j, C.byref(u0), C.byref(u1))
        w0, w1 = B.recycle_uniforms(seed, step, stream, j)
        assert (u0.value, u1.value) == (w0, w1)
        assert 0.0 <= w0 < 1.0 and 0.0 <= w1 < 1.0


def reference_recycle(mk, s, xsize, ysize, vyu, vyl, dt, ttop, tbot, gy_last, mat_plastic, rf, dfric, U):
    """The reference's loops written out in Python (InitializeMarkerRecycling.jl:26-108,
    Extension.jl:53-97, Coordinates.jl:60-127, ResetMarkers.jl:24-268) with rand() taken
    from U(stream, j)."""
    out = {k: np.array(v, copy=True) for k, v in mk.items()}
    air, water, asth = s
    outside = [i for i in range(len(mk["x"])) if mk["inside"][i] != 1]
    nair = sum(1 for i in outside if mk["matid"][i] in (air, water))
    nsub = len(outside) - nair
    newx_air = [0.0 + U(0, j)[0] * xsize for j in range(nair)]
    newy_air = [0.0 + U(0, j)[1] * abs(vyu * dt) for j in range(nair)]
    newx_sub = [0.0 + U(1, j)[0] * xsize for j in range(nsub)]
    newy_sub = [ysize + U(1, j)[1] * -abs(vyl * dt) for j in range(nsub)]
    ia = isub = 0
    idx, flags = [], []
    for i in outside:
        if mk["matid"][i] in (air, water) and nair > 0:
            out["x"][i], out["y"][i] = newx_air[ia], newy_air[ia]
            ia += 1
            flag = 0
        else:
            out["x"][i], out["y"][i] = newx_sub[isub], newy_sub[isub]
            isub += 1
            flag = 1
        idx.append(i + 1)
        flags.append(flag)
    for i, flag in zip(idx, flags):
        i -= 1
        if flag == 0:
            mid, T, P, S, E, V = air, ttop, 0.0, 0.0, 0.0, 0.0
        else:
            mid, T, P, S, E, V = asth, tbot, 3300.0 * 9.81 * gy_last, 1.96e6, 1e-14, 1e20
        out["matid"][i] = mid
        out["tk"][i], out["pr"][i] = T, P
        out["sxx"][i] = out["sxy"][i] = S
        out["exx"][i] = out["exy"][i] = E
        out["sr_ratio"][i] = 0.0
        out["gii"][i] = out["strain_plastic"][i] = out["strain_rate_plastic"][i] = 0.0
        out["meltfrac"][i] = 0.0
        out["eta"][i] = V
        out["pfailure"][i] = np.float32(0.0)
        f = mat_plastic[mid - 1, 2]
        if flag == 1 and rf == 1 and U(2, i)[0] <= 0.5:
            f = f - dfric
        out["fric_ini"][i] = out["fric"][i] = f
    return out, np.array(idx, np.int64), np.array(flags, np.int8), nair


@pytest.mark.parametrize("water,rf", [(1, 0), (2, 1)])
def test_recycle_oracle_matches_reference_loops(eb, B, water, rf):
    rng = np.random.default_rng(21)
    M = 1500
    mk = {k: rng.uniform(-1.0, 1.0, M) for k in B.RECYCLE_FIELDS}
    mk["matid"] = rng.integers(1, 5, M).astype(np.int16)
    mk["pfailure"] = rng.uniform(0, 1, M).astype(np.float32)
    mk["inside"] = np.where(rng.random(M) < 0.9, 1, rng.choice([0, -1], M)).astype(np.int8)
    mp = np.asfortranarray(rng.uniform(0, 1, (4, 6)))
    # sticky air, sticky water, asthenosphere; xsize, ysize, vyu, vyl, dt, T_top, T_bottom, gridy_b[ynum]
    args = (1, water, 4, 500e3, 160e3, -2e-10, 3e-10, 3.15e11, 273.0, 1603.0, 160e3)
    seed, step = 777, 3
    got, idx, fl, nair = B.recycle_extension(mk, *args, mp, rf, 0.05, seed, step)
    want, widx, wfl, wnair = reference_recycle(mk, args[:3], *args[3:11], mp, rf, 0.05,
                                               lambda st, j: B.recycle_uniforms(seed, step, st, j))
    assert nair == wnair and np.array_equal(idx, widx) and np.array_equal(fl, wfl)
    assert len(idx) == int(np.sum(mk["inside"] != 1)) > 0
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        assert np.array_equal(got[k], want[k]), k
    y = got["y"][idx - 1]
    assert np.all(y[fl == 0] >= 0) and np.all(y[fl == 0] < 2e-10 * 3.15e11)
    assert np.all(y[fl == 1] <= 160e3) and np.all(y[fl == 1] > 160e3 - 3e-10 * 3.15e11)


def test_recycle_no_bottom_inflow_oracle_matches_reference_loops(eb, B):
    """ExtensionNoBottomInflow.jl:25-123 written out: outside markers in order, one rand() for
    both coordinates, reset as sticky air."""
    rng = np.random.default_rng(8)
    M = 1200
    mk = {k: rng.uniform(-1.0, 1.0, M) for k in B.RECYCLE_FIELDS}
    mk["matid"] = rng.integers(1, 5, M).astype(np.int16)
    mk["pfailure"] = rng.uniform(0, 1, M).astype(np.float32)
    mk["inside"] = np.where(rng.random(M) < 0.9, 1, -1).astype(np.int8)
    mp = np.asfortranarray(rng.uniform(0, 1, (4, 6)))
    seed, step, vyu, dt = 99, 4, -3e-10, 3.15e11
    got, idx, fl = B.recycle_no_bottom_inflow(mk, 1, 500e3, vyu, dt, 273.0, mp, seed, step)
    want = {k: np.array(v, copy=True) for k, v in mk.items()}
    outside = [i for i in range(M) if mk["inside"][i] != 1]
    for j, i in enumerate(outside):
        u = B.recycle_uniforms(seed, step, 0, j)[0]
        want["y"][i] = u * (vyu * dt)
        want["x"][i] = 0.0 + u * 500e3
        want["matid"][i] = 1
        want["tk"][i] = 273.0
        for k in ("pr", "sxx", "sxy", "exx", "exy", "sr_ratio", "gii", "strain_plastic", "strain_rate_plastic",
                  "meltfrac", "eta"):
            want[k][i] = 0.0
        want["pfailure"][i] = np.float32(0.0)
        want["fric_ini"][i] = want["fric"][i] = mp[0, 2]
    assert np.array_equal(idx, np.array(outside) + 1) and np.all(fl == 0)
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        assert np.array_equal(got[k], want[k]), k


def test_recycle_channel_oracle(B):
    rng = np.random.default_rng(9)
    y = rng.uniform(-5e3, 165e3, 1000)
    tk = rng.uniform(300, 1600, 1000)
    y2, tk2, idx = B.recycle_channel(y, tk, 0.0, 160e3, 273.0, 1603.0)
    moved = y > 160e3
    assert np.array_equal(idx, np.nonzero(moved)[0] + 1)
    assert np.array_equal(y2[moved], y[moved] - 160e3) and np.array_equal(y2[~moved], y[~moved])
    assert np.array_equal(tk2[moved], tk[moved] + 273.0 - 1603.0) and np.array_equal(tk2[~moved], tk[~moved])


def reference_contraction(mk, air, water, layers, strong, xsize, ysize, vfull, dt, h_left, h_right, ttop, thick,
                          x_left, x_right, mat_plastic, rf, dfric, U, asym):
    """ContractionViscoelastic.execute_recycle_steps written out in Python: outside markers in
    order (InitializeMarkerRecycling.jl:26-108), side positions (ContractionRecycleLocations.jl:
    9-140 with CountRecycle.jl:19-29; the y loop and the x loop of Coordinates.jl:223-293 take
    rand() from U(stream, j)[1] and U(stream, j)[0]), the seven-layer and strong-zone material
    of the new position (SevenLayerEarthModel2D.jl:20-62, StrongRegions.jl:24-80) and the
    resets of ResetMarkers.jl:24-268."""
    out = {k: np.array(v, copy=True) for k, v in mk.items()}
    outside = [i for i in range(len(mk["x"])) if mk["inside"][i] != 1]
    nair = sum(1 for i in outside if mk["matid"][i] in (air, water))
    nsub = len(outside) - nair
    disp = abs(vfull) * dt if asym else abs(vfull) * dt * 0.5

    def positions(n, stream, is_air):
        nleft = 0 if asym else n // 2
        newx, newy = [0.0] * n, [0.0] * n
        for start, cnt, h, x0, dx in ((0, nleft, h_left, 0.0, disp), (nleft, n - nleft, h_right, xsize, -disp)):
            y0, yh = (0.0, h) if is_air else (h, ysize - h)
            for j in range(cnt):
                mm = j + start
                newy[mm] = y0 + U(stream, mm)[1] * yh
                newx[mm] = x0 + U(stream, mm)[0] * dx
        return newx, newy

    ax, ay = positions(nair, 0, True)
    sx, sy = positions(nsub, 1, False)
    d = [thick[0]]  # Layers.calc_depths_for_layers: running sums
    for t in thick[1:]:
        d.append(d[-1] + t)

    def material(x, y):
        mid = layers[6]
        if y <= d[0]:
            mid = layers[0]
        else:
            for k in range(1, 6):
                if d[k - 1] < y <= d[k]:
                    mid = layers[k]
                    break
        out_strong = x < x_left or x > x_right
        for k, sid in ((1, strong[0]), (2, strong[1]), (3, strong[2]), (4, strong[2]), (5, strong[2])):
            if d[k - 1] < y <= d[k]:
                if out_strong:
                    mid = sid
                break
        return mid

    ia = isub = 0
    idx, flags = [], []
    for i in outside:
        if mk["matid"][i] in (air, water) and nair > 0:
            out["x"][i], out["y"][i] = ax[ia], ay[ia]
            ia += 1
            flag = 0
        else:
            out["x"][i], out["y"][i] = sx[isub], sy[isub]
            isub += 1
            flag = 1
        idx.append(i + 1)
        flags.append(flag)
    for i, flag in zip(idx, flags):
        i -= 1
        if flag == 0:
            mid, T, P, S, E, V = air, ttop, 0.0, 0.0, 0.0, 0.0
        else:
            mid = material(out["x"][i], out["y"][i])
            T, P, S, E, V = 0.0, 3300.0 * 9.81 * out["y"][i], 1.96e6, 1e-14, 1e20
        out["matid"][i] = mid
        out["tk"][i], out["pr"][i] = T, P
        out["sxx"][i] = out["sxy"][i] = S
        out["exx"][i] = out["exy"][i] = E
        out["sr_ratio"][i] = 0.0
        out["gii"][i] = out["strain_plastic"][i] = out["strain_rate_plastic"][i] = 0.0
        out["meltfrac"][i] = 0.0
        out["eta"][i] = V
        out["pfailure"][i] = np.float32(0.0)
        f = mat_plastic[mid - 1, 2]
        if flag == 1 and rf == 1 and U(2, i)[0] <= 0.5:
            f = f - dfric
        out["fric_ini"][i] = out["fric"][i] = f
    return out, np.array(idx, np.int64), np.array(flags, np.int8), nair


CONTRACTION = dict(layers=(1, 5, 6, 7, 8, 9, 10), strong=(11, 12, 4), thick=(10e3, 15e3, 10e3, 30e3, 20e3, 25e3))


@pytest.mark.parametrize("asym,rf", [(0, 0), (1, 1), (0, 1)])
def test_recycle_contraction_oracle_matches_reference_loops(eb, B, asym, rf):
    rng = np.random.default_rng(31 + asym + 2 * rf)
    M = 3000
    mk = {k: rng.uniform(-1.0, 1.0, M) for k in B.RECYCLE_FIELDS}
    mk["matid"] = rng.integers(1, 13, M).astype(np.int16)
    mk["pfailure"] = rng.uniform(0, 1, M).astype(np.float32)
    mk["inside"] = np.where(rng.random(M) < 0.7, 1, rng.choice([0, -1], M)).astype(np.int8)
    mp = np.asfortranarray(rng.uniform(0, 1, (12, 6)))
    c = CONTRACTION
    xsize, ysize, vfull, dt, hl, hr, ttop = 500e3, 160e3, 3e-9, 3.15e13, 10e3, 12e3, 273.0
    seed, step = 4242, 6
    got, idx, fl, nair = B.recycle_contraction(mk, 1, 2, c["layers"], c["strong"], xsize, ysize, vfull, dt, hl, hr,
                                               ttop, c["thick"], -1.0, 250e3, mp, rf, 0.07, seed, step, asym)
    want, widx, wfl, wnair = reference_contraction(mk, 1, 2, c["layers"], c["strong"], xsize, ysize, vfull, dt, hl,
                                                   hr, ttop, c["thick"], -1.0, 250e3, mp, rf, 0.07,
                                                   lambda st, j: B.recycle_uniforms(seed, step, st, j), asym)
    assert nair == wnair and np.array_equal(idx, widx) and np.array_equal(fl, wfl)
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        assert np.array_equal(got[k], want[k]), k
    # positions: side bands of width |v| dt (/2); the left side (inside the strong-zone limits
    # [-1, 250 km]) takes the seven-layer materials, the right side the strong-zone ones
    x, sub = got["x"][idx - 1], fl == 1
    band = abs(vfull) * dt * (1.0 if asym else 0.5)
    assert np.all((x <= band) | (x >= xsize - band))
    if asym:
        assert np.all(x >= xsize - band)
    ids = set(got["matid"][idx - 1][sub].tolist())
    assert {10, 11, 12, 4}.issubset(ids)
    assert {5, 6, 7, 8, 9}.issubset(ids) == (not asym)


def reference_side_inflow(mk, air, water, asth, xsize, ysize, vyu, dt, ttop, tbot, hl, hr, plate, smooth, vin_l,
                          vin_r, grad, mat_plastic, rf, dfric, U):
    """ExtensionInflowAndOutflowAlongSides.execute_recycling_steps written out in Python
    (ExtensionInflowAndOutflowAlongSides.jl:20-237, Extension.jl:58-73, InflowGeometry.jl,
    InflowRamp.jl, Coordinates.jl:155-200, ResetMarkers.jl:24-268), rand() from U(stream, j)."""
    out = {k: np.array(v, copy=True) for k, v in mk.items()}
    outside = [i for i in range(len(mk["x"])) if mk["inside"][i] != 1]
    nair = sum(1 for i in outside if mk["matid"][i] in (air, water))
    nsub = len(outside) - nair
    newy_air = [0.0 + U(0, j)[1] * abs(vyu * dt) for j in range(nair)]
    newx_air = [0.0 + U(0, j)[0] * xsize for j in range(nair)]
    newx, newy = [0.0] * nsub, [0.0] * nsub
    nleft = nsub // 2
    for start, cnt, h, x0, disp in ((0, nleft, hl, 0.0, abs(vin_l) * dt), (nleft, nsub - nleft, hr, xsize,
                                                                            -abs(vin_r) * dt)):
        y0 = h + plate + smooth
        top, bot = h + plate + smooth, h + plate + smooth + smooth
        for j in range(cnt):
            newy[start + j] = y0 + U(1, start + j)[1] * (ysize - y0)
        for j in range(cnt):
            y = newy[start + j]
            ramp = (y - top) / (bot - top) if top <= y < bot else 1.0
            newx[start + j] = x0 + U(1, start + j)[0] * disp * ramp
    ia = isub = 0
    idx, flags = [], []
    for i in outside:
        if mk["matid"][i] in (air, water) and nair > 0:
            out["x"][i], out["y"][i] = newx_air[ia], newy_air[ia]
            ia += 1
            flag = 0
        else:
            out["x"][i], out["y"][i] = newx[isub], newy[isub]
            isub += 1
            flag = 1
        idx.append(i + 1)
        flags.append(flag)
    for i, flag in zip(idx, flags):
        i -= 1
        if flag == 0:
            mid, T, P, S, E, V = air, ttop, 0.0, 0.0, 0.0, 0.0
        else:
            y = out["y"][i]
            mid, T, P, S, E, V = asth, tbot - grad * ((ysize - y) / 1000.0), 3300.0 * 9.81 * y, 1.96e6, 1e-14, 1e20
        out["matid"][i] = mid
        out["tk"][i], out["pr"][i] = T, P
        out["sxx"][i] = out["sxy"][i] = S
        out["exx"][i] = out["exy"][i] = E
        out["sr_ratio"][i] = 0.0
        out["gii"][i] = out["strain_plastic"][i] = out["strain_rate_plastic"][i] = 0.0
        out["meltfrac"][i] = 0.0
        out["eta"][i] = V
        out["pfailure"][i] = np.float32(0.0)
        f = mat_plastic[mid - 1, 2]
        if flag == 1 and rf == 1 and U(2, i)[0] <= 0.5:
            f = f - dfric
        out["fric_ini"][i] = out["fric"][i] = f
    return out, np.array(idx, np.int64), np.array(flags, np.int8), nair


SIDE_INFLOW = (500e3, 160e3, -2e-10, 3.15e13, 273.0, 1603.0, 10e3, 12e3, 40e3, 15e3, 1e-9, 2e-9, 0.4)


@pytest.mark.parametrize("rf", [0, 1])
def test_recycle_side_inflow_oracle_matches_reference_loops(eb, B, rf):
    rng = np.random.default_rng(61 + rf)
    M = 3000
    mk = {k: rng.uniform(-1.0, 1.0, M) for k in B.RECYCLE_FIELDS}
    mk["matid"] = rng.integers(1, 5, M).astype(np.int16)
    mk["pfailure"] = rng.uniform(0, 1, M).astype(np.float32)
    mk["inside"] = np.where(rng.random(M) < 0.7, 1, rng.choice([0, -1], M)).astype(np.int8)
    mp = np.asfortranarray(rng.uniform(0, 1, (4, 6)))
    seed, step = 1717, 5
    got, idx, fl, nair = B.recycle_side_inflow(mk, 1, 2, 4, *SIDE_INFLOW, mp, rf, 0.03, seed, step)
    want, widx, wfl, wnair = reference_side_inflow(mk, 1, 2, 4, *SIDE_INFLOW, mp, rf, 0.03,
                                                   lambda st, j: B.recycle_uniforms(seed, step, st, j))
    assert nair == wnair and np.array_equal(idx, widx) and np.array_equal(fl, wfl)
    for k in (*B.RECYCLE_FIELDS, "matid", "pfailure"):
        assert np.array_equal(got[k], want[k]), k
    # subsurface markers sit below the inflow top of their side; some inside the ramp
    x, y, sub = got["x"][idx - 1], got["y"][idx - 1], fl == 1
    assert np.all(y[sub] >= 10e3 + 40e3 + 15e3)
    ramp = sub & (y < 12e3 + 40e3 + 30e3) & (y > 12e3 + 40e3 + 15e3)
    assert ramp.sum() > 5


def reference_fz_material(x, y, b, x_start, x_end, ids):
    """FractureZone.define_material (marker_materials/init_manager/types/FractureZone.jl:103-299)."""
    m = ids[6]
    if y <= b[0]:
        m = ids[0]
    if b[0] < y <= b[1]:
        m = ids[1]
    if b[1] < y <= b[2]:
        m = ids[2]
    if b[2] < y <= b[3]:
        m = ids[3]
    if (x < x_end and b[3] < y <= b[4]) or (x >= x_end and b[3] < y <= b[5]):
        m = ids[4]
    if x_start < x < x_end + (b[3] - y) * 25.0 and b[2] < y <= b[3]:
        m = ids[2]
    if x_start < x < x_end and b[3] < y <= b[6]:
        m = ids[5]
    return m


def reference_fz_temperature(y, x, ttop, tbot, grad, x_end, age_l, age_r, sticky, tld_l, tld_r, kappa, ysize):
    """FractureZone.calculate_temperature (temperature/init_manager/types/FractureZone.jl:107-202)."""
    import math

    def lith(asth, depth, age):
        tb = tbot - grad * asth / 1000.0
        return tb + (ttop - tb) * (1 - math.erf(depth / (2 * (kappa * age) ** 0.5)))
    t = tbot - (grad * (ysize - y) / 1000.0)
    if y <= sticky:
        t = ttop
    elif 0 < x < x_end and sticky < y < tld_l:
        t = lith(ysize - tld_l, y - sticky, age_l)
    elif x > x_end and sticky < y < tld_r:
        t = lith(ysize - tld_r, y - sticky, age_r)
    return t


FZ = dict(ids=(1, 5, 6, 7, 8, 9, 10), thick=(10e3, 1e3, 2e3, 4e3, 40e3, 70e3, 20e3), x_start=-1.0, x_end=30e3,
          ages=(10.0, 40.0), tld=(60e3, 100e3), kappa=1e-6, grad=0.4)


@pytest.mark.parametrize("asym", [0, 1])
def test_recycle_fracture_zone_oracle(eb, B, asym):
    """Positions are the contraction ones (the viscoelastic-contraction test pins them); the
    fracture-zone material and temperature of each subsurface marker equal the reference's
    functions written out in Python (temperature within 1e-14: libm's erf against Python's)."""
    rng = np.random.default_rng(81 + asym)
    M = 3000
    mk = {k: rng.uniform(-1.0, 1.0, M) for k in B.RECYCLE_FIELDS}
    mk["matid"] = rng.integers(1, 13, M).astype(np.int16)
    mk["pfailure"] = rng.uniform(0, 1, M).astype(np.float32)
    mk["inside"] = np.where(rng.random(M) < 0.7, 1, rng.choice([0, -1], M)).astype(np.int8)
    mp = np.asfortranarray(rng.uniform(0, 1, (12, 6)))
    z = FZ
    xsize, ysize, vfull, dt, hl, hr, ttop, tbot = 500e3, 160e3, 3e-9, 3.15e13, 10e3, 12e3, 273.0, 1603.0
    seed, step = 5151, 8
    got, idx, fl, nair = B.recycle_fracture_zone(mk, 1, 2, z["ids"], xsize, ysize, vfull, dt, hl, hr, ttop, tbot,
                                                 z["grad"], z["thick"], z["x_start"], z["x_end"], *z["ages"],
                                                 *z["tld"], z["kappa"], mp, 1, 0.02, seed, step, asym)
    ref, ridx, rfl, rnair = B.recycle_contraction(mk, 1, 2, (1,) * 7, (1,) * 3, xsize, ysize, vfull, dt, hl, hr,
                                                  ttop, (1.0,) * 6, -1.0, 1e30, mp, 1, 0.02, seed, step, asym)
    assert nair == rnair and np.array_equal(idx, ridx) and np.array_equal(fl, rfl)
    assert np.array_equal(got["x"], ref["x"]) and np.array_equal(got["y"], ref["y"])
    t = z["thick"]
    b = [t[0]]
    for v in t[1:4]:
        b.append(b[-1] + v)
    b += [b[3] + t[4], b[3] + t[5], b[3] + t[6]]
    spy = 365.25 * 24.0 * 3600.0
    ages = [(a * 1e6) * spy for a in z["ages"]]
    mats, sub = set(), 0
    for i, flag in zip(idx - 1, fl):
        if flag == 0:
            assert got["matid"][i] == 1 and got["tk"][i] == ttop
            continue
        sub += 1
        x, y = got["x"][i], got["y"][i]
        m = reference_fz_material(x, y, b, z["x_start"], z["x_end"], z["ids"])
        assert got["matid"][i] == m
        mats.add(m)
        want_t = reference_fz_temperature(y, x, ttop, tbot, z["grad"], z["x_end"], *ages, t[0], *z["tld"],
                                          z["kappa"], ysize)
        assert abs(got["tk"][i] - want_t) <= 1e-14 * abs(want_t)
        assert got["pr"][i] == 3300.0 * 9.81 * y
        f = mp[m - 1, 2]
        if B.recycle_uniforms(seed, step, 2, i)[0] <= 0.5:
            f = f - 0.02
        assert got["fric"][i] == f
    # (the right side's 12 km sticky layer lies below the sediments' base: no sediment there)
    assert sub > 100 and {6, 7, 8, 10}.issubset(mats) and (5 in mats) == (not asym)


def test_rock_property_laws_match_reference_known_answers(B):
    """The oracle's heat capacity (Waples) and conductivities (Liao14, Sekiguchi-Waples) against
    the reference's own test values (rock_props_tests.jl, tolerance 1e-9 as there)."""
    g, mk, tabs, (nw, nl, ns) = rock_golden_markers()
    cp = B.rock_properties(mk, *tabs, 0, 1, 0, 273.0, 1e30)["rhocp"][:nw]
    np.testing.assert_allclose(cp, g["waples"]["expected_cp"], rtol=0, atol=1e-9)
    k_liao = B.rock_properties(mk, *tabs, 0, 0, 0, 273.0, 1e30)["kt"][nw:nw + nl]
    np.testing.assert_allclose(k_liao, g["liao14"]["expected_k"], rtol=0, atol=1e-9)
    k_sw = B.rock_properties(mk, *tabs, 0, 0, 5, 273.0, 1e30)["kt"][nw + nl:]
    np.testing.assert_allclose(k_sw, g["sekiguchi_waples"]["expected_k"], rtol=0, atol=1e-9)


def test_fracture_zone_erf_law_matches_reference_half_space_cooling(B):
    """The erf law of the oracle's fracture-zone lithosphere temperature, with the mantle base at
    the asthenosphere temperature and age = distance / half spreading rate, against the
    reference's own half-space cooling test values (half_space_cooling_tests.jl, 1e-9)."""
    import json
    import pathlib
    g = json.loads((pathlib.Path(__file__).parent / "golden" / "half_space_reference.json").read_text())
    age = g["distance_from_ridge_meters"] / g["half_spreading_rate_m_s"]
    got = [B.fz_lithosphere_temperature(g["surface_temperature_kelvin"], g["asthenosphere_temperature_kelvin"], 0.0, 0.0,
                                        g["thermal_diffusivity_m2_s"], d, age) for d in g["depths_m"]]
    np.testing.assert_allclose(got, g["expected_temperature_kelvin"], rtol=0, atol=1e-9)
