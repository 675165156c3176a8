"""Calibration table pack: the numeric tables the photon trace reads.

The trace needs the HRMA shell geometry, the iridium optical constants, the
per-shell effective-area correction factors, the WFold scattering tables, the
HETG and LETG grating efficiencies, the grating optical constants (for the
LETG support gratings), the HETG facet sector tables, the ACIS chip corners
the HRC geometry and efficiency tables, and the ACIS sub-pixel offsets of
marx2fits's EDSER pixel adjustment.
MARX reads them at init from its data directory in four formats (RDB text,
big-endian "bdat" float tables, the WFold binary format and FITS binary
tables).  ``build_pack`` reads those files once and writes every table into a
single little-endian ``.mxpack`` file that the C host code maps at
``mx_context_create`` time; the values are bit-for-bit the ones MARX holds in
memory after reading (float32 tables stay float32, RDB numbers are parsed
with correctly rounded decimal conversion like ``sscanf("%lf")``).

Pack layout (all little-endian):
  bytes 0..7    magic ``MXPACK01``
  u32           number of sections
  u32           reserved (0)
  per section:  name (48 bytes, NUL padded), u32 dtype (0 f32, 1 f64, 2 i32),
                u32 ndim, u64 dims[4], u64 offset, u64 nbytes  (= 104 bytes)
  data          each section 64-byte aligned
"""
from __future__ import annotations

import os
import struct
import sys

import numpy as np

MAGIC = b"MXPACK01"
_DT = {0: np.float32, 1: np.float64, 2: np.int32}
_DT_CODE = {np.dtype(np.float32): 0, np.dtype(np.float64): 1, np.dtype(np.int32): 2}
SHELLS = (1, 3, 4, 6)
RDB_COLS = ("x0", "y0", "z0", "p", "k", "rho0", "az_mis", "el_mis", "l")


# ----------------------------------------------------------------- writer --
def write_pack(path: str, sections: dict) -> None:
    names = list(sections)
    hdr_size = 16 + 104 * len(names)
    off = (hdr_size + 63) // 64 * 64
    table, blobs = [], []
    for name in names:
        arr = np.ascontiguousarray(sections[name])
        if arr.dtype not in _DT_CODE:
            raise TypeError(f"{name}: unsupported dtype {arr.dtype}")
        if len(name.encode()) >= 48 or arr.ndim > 4:
            raise ValueError(name)
        dims = list(arr.shape) + [1] * (4 - arr.ndim)
        data = arr.astype(arr.dtype.newbyteorder("<"), copy=False).tobytes()
        table.append(struct.pack("<48sII4QQQ", name.encode(), _DT_CODE[arr.dtype],
                                 arr.ndim, *dims, off, len(data)))
        blobs.append((off, data))
        off = (off + len(data) + 63) // 64 * 64
    buf = bytearray(off)
    buf[0:16] = MAGIC + struct.pack("<II", len(names), 0)
    for i, t in enumerate(table):
        buf[16 + 104 * i:16 + 104 * (i + 1)] = t
    for o, d in blobs:
        buf[o:o + len(d)] = d
    with open(path, "wb") as f:
        f.write(bytes(buf))


def read_pack(path: str) -> dict:
    b = open(path, "rb").read()
    if b[:8] != MAGIC:
        raise ValueError(f"{path}: not a table pack")
    n, _ = struct.unpack_from("<II", b, 8)
    out = {}
    for i in range(n):
        name, dt, nd, d0, d1, d2, d3, off, nb = struct.unpack_from("<48sII4QQQ", b, 16 + 104 * i)
        shape = (d0, d1, d2, d3)[:nd]
        arr = np.frombuffer(b, dtype=np.dtype(_DT[dt]).newbyteorder("<"), count=nb // np.dtype(_DT[dt]).itemsize, offset=off)
        out[name.rstrip(b"\0").decode()] = arr.reshape(shape).astype(_DT[dt])
    return out


# ----------------------------------------------------- MARX format readers --
def read_bdat(path: str) -> np.ndarray:
    """MARX .dat table (marx/data/FORMAT.TXT; reader jdmath/src/bdata.c:80):
    32-byte header (magic 83 43 59 8E, type byte, nrows, ncols, comment
    length), a comment, then nrows rows of ncols big-endian float32."""
    b = open(path, "rb").read()
    if b[:4] != bytes([0x83, 0x43, 0x59, 0x8E]):
        raise ValueError(f"{path}: bad magic")
    if b[4:5] != b"E":
        raise ValueError(f"{path}: not a float32 table")
    nrows, ncols, clen = struct.unpack(">iii", b[5:17])
    data = np.frombuffer(b, dtype=">f4", count=nrows * ncols, offset=32 + clen)
    return data.reshape(nrows, ncols).astype(np.float32).T.copy()      # [col][row]


def read_wfold(path: str):
    """WFold scattering table (marx/libsrc/wfold.c:140-300): repeated records
    of int32 n, six float32 header values and n float32 angles, big-endian.
    Returns (hdr[num,7] f64, theta[num,nmax] f32) sorted by E*sin(alpha) with
    duplicates removed and delta_p recomputed as the reader does."""
    b = open(path, "rb").read()
    off, recs = 0, []
    while off + 4 <= len(b):
        (n,) = struct.unpack_from(">i", b, off)
        if n == 0:
            break
        h = struct.unpack_from(">6f", b, off + 4)
        th = np.frombuffer(b, dtype=">f4", count=n, offset=off + 28).astype(np.float32)
        off += 28 + 4 * n
        e_alpha, p_min, delta_p, p_max, norm, expon = (float(v) for v in h)
        if n == 1:
            p_max = p_min
            delta_p = 0.1
        else:
            delta_p = (p_max - p_min) / float(n - 1)
        recs.append(((e_alpha, p_min, delta_p, p_max, norm, expon, float(n)), th))
    recs.sort(key=lambda r: r[0][0])
    keep = []
    for r in recs:
        if keep and keep[-1][0][0] == r[0][0]:
            raise ValueError(f"{path}: duplicate E*sin(alpha) entries")
        keep.append(r)
    nmax = max(len(r[1]) for r in keep)
    hdr = np.array([r[0] for r in keep], dtype=np.float64)
    theta = np.zeros((len(keep), nmax), dtype=np.float32)
    for i, r in enumerate(keep):
        theta[i, :len(r[1])] = r[1]
    return hdr, theta


def read_rdb(path: str) -> dict:
    """RDB text table (marx/libsrc/rdb.c): '#' comments, a tab-separated
    header line, a column-type line, then rows."""
    lines = [l.rstrip("\n") for l in open(path) if not l.startswith("#") and l.strip()]
    cols = lines[0].split("\t")
    rows = {}
    for l in lines[2:]:
        f = l.split("\t")
        rows[f[0]] = dict(zip(cols, f))
    return rows


def read_column_text(path: str, ncols: int) -> np.ndarray:
    """Whitespace-separated numeric columns, '#' comments (the form read by
    jdmath JDMread_column_ddata)."""
    out = []
    for l in open(path):
        l = l.strip()
        if not l or l.startswith("#"):
            continue
        f = l.split()
        out.append([float(v) for v in f[:ncols]])
    return np.array(out, dtype=np.float64)


def read_simple_data(path: str, names) -> dict:
    """MARX "simple data" text file (_marx_read_simple_data_file,
    marx/libsrc/data.c:334-393): lines "NAME v1 v2 ...", '#' comments; each
    requested name's leading numeric fields, parsed like sscanf("%lf")."""
    want = dict(names)
    out = {}
    for line in open(path):
        f = line.split()
        if not f or f[0].startswith("#") or f[0] not in want:
            continue
        out[f[0]] = [float(v) for v in f[1:1 + want[f[0]]]]
    missing = [k for k in want if k not in out or len(out[k]) != want[k]]
    if missing:
        raise ValueError(f"{path}: missing {missing}")
    return out


# hrc_i_geom.txt fields (hrc_i_geom.c:166-175) and hrc_s_geom.txt fields
# (hrc_s_geom.c:392-413, hrc-s.c:350-360), in the order the pack stores them
HRC_I_GEOM = (("HRC_I_X_Pixel_Size", 1), ("HRC_I_Y_Pixel_Size", 1), ("HRC_I_LL_XYZ", 3), ("HRC_I_Center_XYZ", 3),
              ("HRC_I_LL_to_LR_Vector", 3), ("HRC_I_Center_CXCY", 2), ("HRC_I_Aimpoint_CXCY", 2))
HRC_S_GEOM = (("V_Pixel_Size", 1), ("V_Active", 6), ("U_Pixel_Size", 1), ("U_Active", 2), ("Aimpoint_Offset", 3),
              ("Left_UV", 2), ("Right_UV", 2), ("Middle_UV", 2), ("Left_XYZ", 3), ("Right_XYZ", 3),
              ("Middle_XYZ", 3), ("Left_CXCY", 2), ("Right_CXCY", 2), ("Middle_CXCY", 2), ("Left_Angle", 1),
              ("Right_Angle", 1), ("Detector_Angle", 1), ("Ion_Shield_T", 1), ("Ion_Shield_L", 1),
              ("Ion_Shield_R", 1), ("Ion_Shield_X", 1), ("Ion_Shield_SL", 1), ("Ion_Shield_SR", 1),
              ("Ion_Shield_GapL", 1), ("Ion_Shield_GapR", 1))


def read_fits_bintables(path: str):
    """Minimal FITS reader: yields (header dict, {column: ndarray}) for each
    BINTABLE extension.  Handles the scalar/vector numeric (E, D, J, I, K, B),
    character (A) and bit (X, as bytes) columns the CALDB files and event
    lists use."""
    b = open(path, "rb").read()
    off, hdus = 0, []
    while off < len(b):
        hdr = {}
        while True:
            blk = b[off:off + 2880]
            if len(blk) < 2880:
                raise ValueError(f"{path}: truncated FITS header")
            off += 2880
            done = False
            for i in range(36):
                c = blk[i * 80:(i + 1) * 80].decode("ascii", "replace")
                k = c[:8].strip()
                if k == "END":
                    done = True
                    break
                if c[8:10] == "= ":
                    v = c[10:]
                    if v.lstrip().startswith("'"):
                        v = v.lstrip()[1:]
                        v = v[:v.index("'")].rstrip()
                    else:
                        v = v.split("/")[0].strip()
                    hdr[k] = v
            if done:
                break
        naxis = int(hdr.get("NAXIS", "0"))
        size = 0
        if naxis > 0:
            size = 1
            for i in range(1, naxis + 1):
                size *= int(hdr[f"NAXIS{i}"])
            size = size * abs(int(hdr["BITPIX"])) // 8 + int(hdr.get("PCOUNT", "0"))
        data_off = off
        off += (size + 2879) // 2880 * 2880
        if hdr.get("XTENSION") != "BINTABLE":
            continue
        rowlen, nrows = int(hdr["NAXIS1"]), int(hdr["NAXIS2"])
        raw = b[data_off:data_off + rowlen * nrows]
        cols, pos = {}, 0
        for i in range(1, int(hdr["TFIELDS"]) + 1):
            form = hdr[f"TFORM{i}"].strip()
            j = 0
            while j < len(form) and form[j].isdigit():
                j += 1
            rep = int(form[:j]) if j else 1
            code = form[j]
            sz = {"E": 4, "D": 8, "J": 4, "I": 2, "A": 1, "K": 8, "B": 1, "X": 1}[code]
            name = hdr[f"TTYPE{i}"].strip()
            if code == "X":   # bit array: its bytes, rows x ceil(rep / 8)
                rep = (rep + 7) // 8
                vals = np.array([np.frombuffer(raw, dtype=np.uint8, count=rep, offset=r * rowlen + pos)
                                 for r in range(nrows)]).reshape(nrows, rep)
            elif code == "A":
                vals = [raw[r * rowlen + pos:r * rowlen + pos + rep].decode().rstrip(" \0") for r in range(nrows)]
            else:
                dt = {"E": ">f4", "D": ">f8", "J": ">i4", "I": ">i2", "K": ">i8", "B": ">u1"}[code]
                a = np.empty((nrows, rep), dtype=dt)
                for r in range(nrows):
                    a[r] = np.frombuffer(raw, dtype=dt, count=rep, offset=r * rowlen + pos)
                vals = a.astype(dt[1:]) if rep > 1 else a[:, 0].astype(dt[1:])
            cols[name] = vals
            pos += rep * sz
        hdus.append((hdr, cols))
    return hdus


def read_fef(path: str) -> dict:
    """The acis/fef sections from an ACIS FEF file (its FUNCTION table, as
    read_fef_file reads it, acis_fef.c:819-874): rows = CCD_ID, CHIPX_LO,
    CHIPX_HI, CHIPY_LO, CHIPY_HI, REGNUM; vals = ENERGY, CHANNEL, then
    G<k>_FWHM, G<k>_POS, G<k>_AMPL for each gaussian the file has, in row
    order."""
    for h, c in read_fits_bintables(path):
        if h.get("EXTNAME", "").upper() != "FUNCTION":
            continue
        cols = {k.upper(): v for k, v in c.items()}
        ng = 0
        while all(f"G{ng + 1}_{x}" in cols for x in ("FWHM", "POS", "AMPL")):
            ng += 1
        rows = np.stack([np.asarray(cols[k]) for k in ("CCD_ID", "CHIPX_LO", "CHIPX_HI", "CHIPY_LO", "CHIPY_HI",
                                                       "REGNUM")], axis=1).astype(np.int32)
        vals = [cols["ENERGY"], cols["CHANNEL"]] + [cols[f"G{k + 1}_{x}"] for k in range(ng)
                                                    for x in ("FWHM", "POS", "AMPL")]
        return {"acis/fef/rows": rows, "acis/fef/vals": np.stack([np.asarray(v) for v in vals], axis=1).astype(np.float32)}
    raise ValueError(f"{path}: no FUNCTION table")


def read_contam(path: str) -> dict:
    """The acis/contam<ccd>/* sections from an ACIS contamination file
    (read_contam_file_for_ccd, aciscontam.c:315-487): per chip extension
    ACIS<ccd>_CONTAM (or AXAF_CONTAM with CCD_ID), one row per layer:
    rows = (component, n_energy, n_time), energy and mu [layer][repeat],
    time [layer][repeat] (double), tau0 and tau1, and the optional fxy map
    with its blocking factor fxyblk."""
    S = {}
    for h, c in read_fits_bintables(path):
        ext = h.get("EXTNAME", "").upper()
        if ext.startswith("ACIS") and ext.endswith("_CONTAM") and ext[4:-7].isdigit():
            ccd = int(ext[4:-7])
        elif ext == "AXAF_CONTAM" and "CCD_ID" in h:
            ccd = int(h["CCD_ID"])
        else:
            continue
        cols = {k.lower(): v for k, v in c.items()}
        two = lambda a: np.asarray(a).reshape(len(np.asarray(a)), -1)
        k = f"acis/contam{ccd}/"
        S[k + "rows"] = np.stack([np.asarray(cols["component"]), np.asarray(cols["n_energy"]),
                                  np.asarray(cols["n_time"])], axis=1).astype(np.int32)
        S[k + "energy"] = two(cols["energy"]).astype(np.float32)
        S[k + "mu"] = two(cols["mu"]).astype(np.float32)
        S[k + "time"] = two(cols["time"]).astype(np.float64)
        S[k + "tau0"] = two(cols["tau0"]).astype(np.float32)
        S[k + "tau1"] = two(cols["tau1"]).astype(np.float32)
        if "fxy" in cols:
            S[k + "fxy"] = two(cols["fxy"]).astype(np.float32)
            S[k + "fxyblk"] = np.array([int(h.get("FXYBLK", "1"))], dtype=np.int32)
    if not S:
        raise ValueError(f"{path}: no ACIS contamination tables")
    return S


def pack_with_fef(pack_in: str, fef_path: str, pack_out: str, contam_path: str | None = None) -> None:
    """A copy of a table pack with the ACIS FEF of fef_path (and the ACIS
    contamination file contam_path) added."""
    S = read_pack(pack_in)
    S.update(read_fef(fef_path))
    if contam_path:
        S.update(read_contam(contam_path))
    write_pack(pack_out, S)


# ---------------------------------------------------------------- builder --
def build_sections(data_dir: str) -> dict:
    """Collect every table from a MARX data directory (marx/data)."""
    S = {}
    rdb = read_rdb(os.path.join(data_dir, "hrma", "EKCHDOS06.rdb"))
    geo = np.zeros((8, len(RDB_COLS)), dtype=np.float64)
    for j, kind in enumerate("ph"):
        for i, s in enumerate(SHELLS):
            row = rdb[f"{kind}{s}"]
            geo[4 * j + i] = [float(row[c]) for c in RDB_COLS]
    S["hrma/rdb"] = geo
    S["hrma/optconst"] = read_bdat(os.path.join(data_dir, "hrma", "iridium.dat"))[:3]
    for s in SHELLS:
        S[f"hrma/corr{s}"] = read_bdat(os.path.join(data_dir, "hrma", f"corr_{s}.dat"))[:2]
    for kind in "ph":
        for s in SHELLS:
            hdr, theta = read_wfold(os.path.join(data_dir, "hrma", f"scat_{kind}{s}_M.bin"))
            S[f"wfold/{kind}{s}/hdr"] = hdr
            S[f"wfold/{kind}{s}/theta"] = theta

    geff = read_fits_bintables(os.path.join(data_dir, "caldb", "hetgD1996-11-01greffpr001N0007.fits"))
    byname = {h.get("HDUNAME", ""): c for h, c in geff}
    for i in range(4):
        c = byname[f"AXAF_GREFF{i + 1}"]
        S[f"hetg/geff{i}/energy"] = np.asarray(c["ENERGY"], dtype=np.float32)
        S[f"hetg/geff{i}/eff"] = np.ascontiguousarray(np.asarray(c["EFF"], dtype=np.float32).T)
    geff = read_fits_bintables(os.path.join(data_dir, "caldb", "letgD1996-11-01greffpr001N0007.fits"))
    byname = {h.get("HDUNAME", ""): c for h, c in geff}
    for i in range(4):
        c = byname[f"AXAF_GREFF{i + 1}"]
        S[f"letg/geff{i}/energy"] = np.asarray(c["ENERGY"], dtype=np.float32)
        S[f"letg/geff{i}/eff"] = np.ascontiguousarray(np.asarray(c["EFF"], dtype=np.float32).T)
    # energy, beta, delta and the transmissions of gold, polyimide, chromium
    # and nickel (read_grating_optical_consts, diffract.c:195-258)
    S["grating/optconst"] = read_bdat(os.path.join(data_dir, "grating", "optical-constants.dat"))
    sector_files = {1: "hetgmp1D1996-11-01marxsectorN0002.tbl", 3: "hetgmp3D1996-11-01marxsectorN0002.tbl",
                    4: "hetgmp4D1996-11-01marxsectorN0003.tbl", 6: "hetgmp6D1996-11-01marxsectorN0003.tbl"}
    for s, fn in sector_files.items():
        S[f"hetg/sector{s}"] = read_column_text(os.path.join(data_dir, "grating", fn), 6)

    geom = read_fits_bintables(os.path.join(data_dir, "caldb", "telD1999-07-23geomN0006.fits"))
    for h, c in geom:
        if h.get("EXTNAME") == "INSTGEOM" and h.get("INSTRUME") == "ACIS":
            ids = np.asarray(c["CHIP_ID"], dtype=np.float64)[:, None]
            S["acis/geom"] = np.hstack([ids, c["LL"], c["LR"], c["UL"], c["UR"]]).astype(np.float64)
        if h.get("EXTNAME") == "INSTRUMENTS":
            k = [n.strip().upper() for n in c["INSTRUMENT"]].index("ACIS")
            S["acis/origin"] = np.asarray(c["ORIGIN"][k], dtype=np.float64)
    aim = read_fits_bintables(os.path.join(data_dir, "caldb", "telD1999-07-23aimptsN0002.fits"))
    for h, c in aim:
        if h.get("EXTNAME") == "AIMPOINTS":
            names = [n.strip().upper() for n in c["AIMPOINT_NAME"]]
            S["acis/aimpt_i"] = np.asarray(c["AIMPOINT"][names.index("AI2")], dtype=np.float64)
            S["acis/aimpt_s"] = np.asarray(c["AIMPOINT"][names.index("AS1")], dtype=np.float64)
    # HRC: geometry, CALDB origins and aimpoints, MCP and UV/ion shield
    # efficiencies (marx.par defaults), Drake flat optical constants
    for key, fname, fields in (("hrc/i_geom", "hrc_i_geom.txt", HRC_I_GEOM), ("hrc/s_geom", "hrc_s_geom.txt", HRC_S_GEOM)):
        v = read_simple_data(os.path.join(data_dir, "hrc", fname), fields)
        S[key] = np.array([x for k, _ in fields for x in v[k]], dtype=np.float64)
    for h, c in geom:
        if h.get("EXTNAME") == "INSTRUMENTS":
            names = [n.strip().upper() for n in c["INSTRUMENT"]]
            S["hrc/origin_i"] = np.asarray(c["ORIGIN"][names.index("HRC-I")], dtype=np.float64)
            S["hrc/origin_s"] = np.asarray(c["ORIGIN"][names.index("HRC-S")], dtype=np.float64)
    for h, c in aim:
        if h.get("EXTNAME") == "AIMPOINTS":
            names = [n.strip().upper() for n in c["AIMPOINT_NAME"]]
            S["hrc/aimpt_i"] = np.asarray(c["AIMPOINT"][names.index("HI1")], dtype=np.float64)
            S["hrc/aimpt_s"] = np.asarray(c["AIMPOINT"][names.index("HS1")], dtype=np.float64)
    for key, fname in (("hrc/qe_i", "mcp_qe_i.v2.2.dat"), ("hrc/uvis_i", "uvis_i.v4.dat"),
                       ("hrc/qe_s", "mcp_qe_s.v3.dat"), ("hrc/uvis_s0", "uvis_s1.v4.dat"),
                       ("hrc/uvis_s1", "uvis_s2.v4.dat"), ("hrc/uvis_s2", "uvis_s56.v4.dat"),
                       ("hrc/uvis_s3", "uvis_s34.v4.dat")):
        S[key] = read_bdat(os.path.join(data_dir, "hrc", fname))[:2]
    S["hrc/optconst_cr"] = read_bdat(os.path.join(data_dir, "hrc", "chromium.dat"))[:3]
    S["hrc/optconst_c"] = read_bdat(os.path.join(data_dir, "hrc", "carbon.dat"))[:3]
    # ACIS sub-pixel event positions (read_subpix_ext, acis_subpix.c:96-186):
    # per flight grade its number of points, then energies, CHIPX and CHIPY
    # offsets padded to the column's repeat count
    sub = read_fits_bintables(os.path.join(data_dir, "caldb", "acisD1999-07-22subpixN0001_marx.fits"))
    for h, c in sub:
        kind = {"MARX_ACIS_SUBPIX_FI": "fi", "MARX_ACIS_SUBPIX_BI": "bi"}.get(h.get("EXTNAME"))
        if kind is None:
            continue
        cols = {k.upper(): v for k, v in c.items()}
        S[f"acis/subpix_{kind}/rows"] = np.stack([cols["FLTGRADE"], cols["NPOINTS"]], axis=1).astype(np.int32)
        S[f"acis/subpix_{kind}/table"] = np.stack([cols["ENERGY"], cols["CHIPX_OFFSET"],
                                                   cols["CHIPY_OFFSET"]]).astype(np.float32)
    fef = os.path.join(data_dir, "caldb", "acisfef.fits")     # the ACISFEF entry of marxcaldb.par
    if os.path.exists(fef):
        S.update(read_fef(fef))
    contam = os.path.join(data_dir, "caldb", "acisD1999-08-13contamN0015_marx.fits")   # ACISCONTAM
    if os.path.exists(contam):
        S.update(read_contam(contam))
    qe = read_fits_bintables(os.path.join(data_dir, "caldb", "acisD1997-04-17qeN0006.fits"))
    for h, c in qe:
        if h.get("EXTNAME") == "AXAF_QE":
            S[f"acis/qe{int(h['CCD_ID'])}"] = np.vstack([c["ENERGY"], c["QE"]]).astype(np.float32)
    # the parameter file marx ships (marx/par/marx.par): the template of a
    # run's parameter file
    par = os.path.join(data_dir, os.pardir, "par", "marx.par")
    if os.path.exists(par):
        S["par/marx"] = text_section(open(par, "rb").read())
    # the observation templates obs.par of a run starts from (write_obs_par,
    # marx.c:999-1196), as text sections
    obs_dir = os.path.join(data_dir, "obs")
    for f in sorted(os.listdir(obs_dir)) if os.path.isdir(obs_dir) else []:
        if f.endswith(".par"):
            S[f"obs/{f[:-4]}"] = text_section(open(os.path.join(obs_dir, f), "rb").read())
    return S


def text_section(b: bytes) -> np.ndarray:
    """Bytes as an int32 section: the byte count, then the bytes four to a
    word (little-endian), zero padded."""
    pad = b + b"\0" * (-len(b) % 4)
    return np.concatenate([np.array([len(b)], dtype=np.int32), np.frombuffer(pad, dtype="<i4").astype(np.int32)])


def section_text(a: np.ndarray) -> bytes:
    return a[1:].astype("<i4").tobytes()[: int(a[0])]


DEFAULT_PACK = os.path.join(os.path.dirname(os.path.abspath(__file__)), "marx_tables.mxpack")


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="Build the table pack from a MARX data directory")
    ap.add_argument("marx_data_dir", help="MARX data directory (the one holding hrma/, grating/, caldb/)")
    ap.add_argument("-o", "--output", default=DEFAULT_PACK)
    a = ap.parse_args(argv)
    S = build_sections(a.marx_data_dir)
    write_pack(a.output, S)
    print(f"wrote {a.output}: {len(S)} sections, {os.path.getsize(a.output)} bytes")


if __name__ == "__main__":
    sys.exit(main())
