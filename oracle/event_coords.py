"""CPU restatement of marx2fits's per-event coordinates (test infrastructure).

Only the tests and fixture scripts use this module; it is the checker of the
device event pass (``mx_event_coords``), never a code path of the product.
It restates, with numpy float64 in the reference's order of operations,

  read_float32_add_1      marx/src/marx2fits.c:3460-3470   CHIPX, CHIPY
  compute_expno           marx/src/marx2fits.c:3741-3761   EXPNO, frame starts
  read_dither_value       marx/src/marx2fits.c:3567-3581   dither of the frame
  compute_fltgrade/grade  marx/src/marx2fits.c:3813-3866   FLTGRADE, GRADE
  compute_detxy           marx/src/marx2fits.c:3676-3736   DETX, DETY
    marx_init_chip_to_mnc, marx_chip_to_mnc   marx/libsrc/pixlib.c:135-222
    marx_mnc_to_fpc                            marx/libsrc/detpix.c:182-208
    marx_compute_acis_subpix                   marx/libsrc/acis_subpix.c:284-320
  compute_xy_sky          marx/src/marx2fits.c:3869-3910   X, Y
    unapply_dither                             marx/libsrc/dither.c:583-607
    marx_mnc_to_ra_dec, marx_compute_ra_dec_offsets  marx/libsrc/pixlib.c:499-570
  compute_tdetxy          marx/src/marx2fits.c:3584-3598   TDETX, TDETY
    acis_i_to_tiled, acis_s_to_tiled  marx/libsrc/acis_geom.c:106-203
    hrc_i_to_tiled, hrc_s_to_tiled    marx/libsrc/hrc_i_geom.c:215-233, hrc_s_geom.c:476-514

and the jdmath vector primitives JDMv_length, JDMv_normalize and
JDMv_rotate_vector1 (jdmath/src/vector.c:77-109, 187-206).  The facet
geometry is the reference's own (``mxref_detector_geometry``,
``mxref_facet_tdet``, ``mxref_fp_system``), stored with each fixture.

Pinned against the reference's marx2fits program (compiled from its sources
with a file-served JDMrandom, oracle/Makefile target m2f) on the events of
``tests/golden/events_*.npz``: equal single-precision outputs.
"""
from __future__ import annotations

import numpy as np

EXACT, NONE, RANDOMIZE, EDSER = 3, 2, 1, 0
PIXADJ = {"EDSER": EDSER, "RANDOMIZE": RANDOMIZE, "NONE": NONE, "EXACT": EXACT}

# Flight_Grade_Table (marx2fits.c:3838-3849): 3 x 3 sub-pixels, four grades each
FLIGHT_GRADES = np.array([[10, 11, 138, 139], [2, 34, 130, 162], [18, 22, 50, 54],
                          [8, 12, 136, 140], [0, 0, 0, 0], [16, 17, 48, 49],
                          [72, 76, 104, 108], [64, 65, 68, 69], [80, 81, 208, 209]], dtype=np.int16)
# Grade_Map (marx2fits.c:3792-3810), one digit per flight grade
GRADE_MAP = np.array([int(c) for c in
                      "0125115735663577446755677777777711251157577757774467556777777777"
                      "2277227767776777667777777777777755775577677767777777777777777777"
                      "1125115735663577557777777777777711251157577757775577777777777777"
                      "5577557777777777667777777777777777777777777777777777777777777777"], dtype=np.int16)


def jdm_length(x, y, z):
    """JDMv_length (vector.c:77-97), elementwise."""
    x, y, z = np.abs(x), np.abs(y), np.abs(z)
    c = z < x
    z, x = np.where(c, x, z), np.where(c, z, x)
    c = z < y
    z, y = np.where(c, y, z), np.where(c, z, y)
    with np.errstate(invalid="ignore", divide="ignore"):
        x = x / z
        y = y / z
        r = z * np.sqrt(1.0 + x * x + y * y)
    return np.where(z == 0.0, 0.0, r)


def jdm_normalize(v):
    ln = jdm_length(*v)
    with np.errstate(invalid="ignore", divide="ignore"):
        return [np.where(ln != 0.0, c / ln, c) for c in v]


def jdm_rotate_unit(p, n, c, s):
    """JDMv_rotate_unit_vector1 (vector.c:187-206): Rodrigues, then normalised."""
    pn = p[0] * n[0] + p[1] * n[1] + p[2] * n[2]
    b = pn * (1.0 - c)
    cz = n[0] * p[1] - n[1] * p[0]
    cx = n[1] * p[2] - n[2] * p[1]
    cy = n[2] * p[0] - n[0] * p[2]
    return jdm_normalize([c * p[0] + b * n[0] + s * cx, c * p[1] + b * n[1] + s * cy,
                          c * p[2] + b * n[2] + s * cz])


def jdm_bsearch_f(x, xp):
    """JDMbinary_search_f (finterpo.c:37-57) for one float32 table, many x."""
    x = np.asarray(x, dtype=np.float32)
    n = len(xp)
    n0 = np.zeros(x.shape, dtype=np.int64)
    n1 = np.full(x.shape, n, dtype=np.int64)
    done = np.zeros(x.shape, dtype=bool)
    out = np.zeros(x.shape, dtype=np.int64)
    while True:
        act = ~done & (n1 > n0 + 1)
        if not act.any():
            break
        n2 = (n0 + n1) // 2
        v = xp[np.minimum(n2, n - 1)]
        ge = act & (v >= x)
        eq = ge & (v == x)
        out[eq] = n2[eq]
        done |= eq
        n1 = np.where(ge & ~eq, n2, n1)
        n0 = np.where(act & ~ge, n2, n0)
    rest = ~done
    out[rest] = np.where(x[rest] >= xp[n0[rest]], n1[rest], n0[rest])
    return out


def subpix(tables, ccd, energy, fltgrade):
    """marx_compute_acis_subpix (acis_subpix.c:284-320): float32 dx, dy.
    tables: {"fi"|"bi": {fltgrade: (energies, dxs, dys)}}."""
    dx = np.zeros(len(ccd), dtype=np.float32)
    dy = np.zeros(len(ccd), dtype=np.float32)
    kind = np.where((ccd == 5) | (ccd == 7), 1, 0)
    for kd, name in enumerate(("fi", "bi")):
        for fg, (e, xs, ys) in tables[name].items():
            m = (kind == kd) & (fltgrade == fg)
            if not m.any():
                continue
            en = np.asarray(energy, dtype=np.float32)[m]
            nn = len(e)
            j = jdm_bsearch_f(en, e)
            j = np.where(j == 0, 1, j)
            j = np.where(j == nn, j - 1, j)
            e0, e1 = e[j - 1], e[j]
            w1 = (en.astype(np.float64) - e0.astype(np.float64)) / (e1 - e0).astype(np.float64)
            w0 = 1.0 - w1
            dx[m] = (w0 * xs[j - 1].astype(np.float64) + w1 * xs[j].astype(np.float64)).astype(np.float32)
            dy[m] = (w0 * ys[j - 1].astype(np.float64) + w1 * ys[j].astype(np.float64)).astype(np.float32)
    return dx, dy


def subpix_tables(pack_sections):
    """The sub-pixel rows of a table pack (acis/subpix_{fi,bi})."""
    out = {}
    for name in ("fi", "bi"):
        rows = pack_sections[f"acis/subpix_{name}/rows"]
        tab = pack_sections[f"acis/subpix_{name}/table"]
        d = {}
        for r, (fg, npts) in enumerate(rows):
            if npts > 0:
                d[int(fg)] = (tab[0, r, :npts].copy(), tab[1, r, :npts].copy(), tab[2, r, :npts].copy())
        out[name] = d
    return out


def event_coords(detector, geom, tdet, fp, params, ev, uniforms, sub=None):
    """Columns of marx2fits for one event list.

    geom    (nfacets, 20): mxref_detector_geometry rows (id, x_ll, xhat, yhat,
            normal, xlen, ylen, x_pixel_size, y_pixel_size, xpixel_offset,
            ypixel_offset, 0)
    tdet    (nfacets, 2): tdet_xoff, tdet_yoff; fp: fp_delta_s0, fp_x0, fp_y0
    detector "ACIS-I", "ACIS-S", "HRC-I" or "HRC-S"
    params  dict: focal_length, det_offset (3), roll_nom (deg), frame_time,
            dithered, pixel_adjust (EXACT/NONE/RANDOMIZE/EDSER)
    ev      dict of columns: ccd (int), xpixel, ypixel, time (float32),
            sky_ra, sky_dec, sky_roll, det_dy, det_dz, det_theta (float32),
            b_energy (float32)
    uniforms (3, n): grade draw, x and y randomisation
    """
    n = len(ev["ccd"])
    acis = detector.startswith("ACIS")
    ccd = np.asarray(ev["ccd"]).astype(np.int64)
    fi = ccd - int(geom[0, 0])
    if (fi < 0).any() or (fi >= len(geom)).any():
        raise ValueError("chip id outside the detector")
    g = geom[fi]
    padj = params["pixel_adjust"]
    if not acis and padj == EDSER:
        padj = RANDOMIZE
    f32 = np.float32
    chipx = (np.asarray(ev["xpixel"], f32) + f32(1.0)).astype(f32)
    chipy = (np.asarray(ev["ypixel"], f32) + f32(1.0)).astype(f32)
    t = np.asarray(ev["time"], f32).astype(np.float64)
    k = np.arange(n)
    # EXPNO and the frame whose first event's dither state an event uses
    if acis and params["frame_time"] > 0:
        expno = np.trunc(t / params["frame_time"]).astype(np.int64)
        prev = np.concatenate([[-1], expno[:-1]])
        update = expno != prev
    else:
        expno = (k - 1).astype(np.int64)
        update = np.ones(n, dtype=bool)
    if not acis or padj == EXACT:
        update = np.ones(n, dtype=bool)
    first = np.maximum.accumulate(np.where(update, k, 0))
    d = {}
    for c in ("sky_ra", "sky_dec", "sky_roll", "det_dy", "det_dz", "det_theta"):
        v = np.asarray(ev[c], f32).astype(np.float64) if params["dithered"] else np.zeros(n)
        d[c] = v[first]
    # FLTGRADE, GRADE
    u = np.asarray(uniforms, dtype=np.float64).reshape(3, n)
    fltgrade = np.zeros(n, dtype=np.int16)
    if acis:
        cx, cy = chipx.astype(np.float64), chipy.astype(np.float64)
        sx = (3.0 * (cx - np.floor(cx))).astype(np.int64)
        sy = (3.0 * (cy - np.floor(cy))).astype(np.int64)
        fltgrade = FLIGHT_GRADES[3 * sy + sx, np.minimum((4 * u[0]).astype(np.int64), 3)]
    grade = GRADE_MAP[fltgrade.astype(np.int64) & 0xFF] if acis else np.zeros(n, np.int16)
    # DETX, DETY
    x = chipx.astype(np.float64) - 1.0
    y = chipy.astype(np.float64) - 1.0
    if padj == NONE:
        x, y = np.floor(x) + 0.5, np.floor(y) + 0.5
    elif padj == RANDOMIZE:
        x, y = np.floor(x) + u[1], np.floor(y) + u[2]
    elif padj == EDSER:
        dx, dy = subpix(sub, ccd, np.asarray(ev["b_energy"], f32), fltgrade)
        x = np.floor(x) + 0.5 + dx.astype(np.float64)
        y = np.floor(y) + 0.5 + dy.astype(np.float64)
    th = d["det_theta"]
    ct, st = np.cos(th), np.sin(th)
    F = params["focal_length"]
    off = params["det_offset"]
    ll, xh, yh = g[:, 1:4].T, g[:, 4:7].T, g[:, 7:10].T
    xps, yps, xoff, yoff = g[:, 15], g[:, 16], g[:, 17], g[:, 18]
    yo = off[1] + d["det_dy"]
    zo = off[2] + d["det_dz"]
    ofs = [np.full(n, off[0] - F), yo + ct * ll[1] - st * ll[2], zo + st * ll[1] + ct * ll[2]]
    e1 = [xh[0], ct * xh[1] - st * xh[2], st * xh[1] + ct * xh[2]]
    e2 = [yh[0], ct * yh[1] - st * yh[2], st * yh[1] + ct * yh[2]]
    e1 = [xps * c for c in e1]
    e2 = [yps * c for c in e2]
    xp, yp = x - xoff, y - yoff
    mnc = jdm_normalize([ofs[i] + e1[i] * xp + e2[i] * yp for i in range(3)])
    delta, x0, y0 = fp
    with np.errstate(divide="ignore", invalid="ignore"):
        factor = 1.0 / (delta * mnc[0])
    detx = x0 - factor * mnc[1]
    dety = y0 + factor * mnc[2]
    # X, Y
    if not params["dithered"]:
        th = params["roll_nom"] * np.pi / 180.0
        c, s = np.cos(th), np.sin(th)
        ddx, ddy = detx - x0, dety - y0
        X = x0 + c * ddx + s * ddy
        Y = y0 - s * ddx + c * ddy
    else:
        ra, dec, roll = d["sky_ra"], d["sky_dec"], d["sky_roll"]
        cra, sra, cdec, sdec = np.cos(ra), np.sin(ra), np.cos(dec), np.sin(dec)
        cos_t = cdec * cra
        nv = [np.zeros(n), -sdec, cdec * sra]
        sin_t = jdm_length(*nv)
        big = sin_t >= 1e-20
        with np.errstate(divide="ignore", invalid="ignore"):
            nv = [c / sin_t for c in nv]
        rot = jdm_rotate_unit(mnc, nv, cos_t, sin_t)
        p = [np.where(big, rot[i], mnc[i]) for i in range(3)]
        ones, zeros = np.ones(n), np.zeros(n)
        p = jdm_rotate_unit(p, [ones, zeros, zeros], np.cos(roll), np.sin(roll))
        perp = np.sqrt(p[0] * p[0] + p[1] * p[1])
        perp = np.minimum(perp, 1.0)
        dec_s = np.where(p[2] <= 0, np.arccos(perp), -np.arccos(perp))
        q = -p[0] / perp
        ra_s = np.where(p[1] <= 0.0, np.arccos(q), -np.arccos(q))
        cd = np.cos(dec_s)
        fac = cd * (1 - np.cos(ra_s))
        sdd = np.sin(dec_s) + fac * 0.0
        sdd = np.where(np.abs(sdd) > 1.0, np.sign(sdd), sdd)
        ddec = np.arcsin(sdd)
        num = cd * np.sin(ra_s)
        den = np.cos(dec_s) - fac * 1.0
        a = np.arctan(num / den)
        dra = np.where(den >= 0, a, np.where(num >= 0, a + np.pi, a - np.pi))
        X = -dra / delta + x0
        Y = ddec / delta + y0
    # TDETX, TDETY
    ix = chipx.astype(np.uint32).astype(np.float64)
    iy = chipy.astype(np.uint32).astype(np.float64)
    tdx, tdy = tdet[fi, 0], tdet[fi, 1]
    if detector == "ACIS-I":
        a02 = (ccd == 0) | (ccd == 2)
        xf = np.where(a02, tdx + iy, tdx - iy)
        yf = np.where(a02, tdy - ix, tdy + ix)
    else:
        xf, yf = ix + tdx, iy + tdy
    xf = np.maximum(xf.astype(np.float32), 0).astype(np.uint32) + 1
    yf = np.maximum(yf.astype(np.float32), 0).astype(np.uint32) + 1
    return dict(chipx=chipx, chipy=chipy, expno=(expno if acis else np.zeros(n, np.int64)).astype(np.int32),
                fltgrade=fltgrade.astype(np.int16), grade=grade.astype(np.int16), detx=detx, dety=dety,
                x=X, y=Y, tdetx=xf.astype(np.int32), tdety=yf.astype(np.int32))
