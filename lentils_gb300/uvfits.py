"""uvfits (FITS random groups) visibility loader, restating the reference's
``_load_uvfits`` (lentils/common/data_util.py:5-76) without astropy.

A FITS file is a sequence of HDUs: 2880-byte blocks of 80-character header cards ending in
END, then big-endian data padded to 2880 bytes. The primary HDU of a uvfits file holds random
groups (GROUPS = T, NAXIS1 = 0): GCOUNT groups of PCOUNT parameters (UU, VV, WW, DATE, ...,
each scaled by PSCALn / PZEROn, parameters of the same name summed) followed by an array
of NAXIS2 x ... x NAXISn values (COMPLEX = re, im, weight fastest, then STOKES, FREQ, IF, RA,
DEC). The 'AIPS FQ' binary table gives each IF's frequency offset and channel width.

load_uvfits returns what the reference's loader returns: the visibility space (channels in Hz
= CH WIDTH x (channel - reference channel) + IF FREQ + reference frequency, for all IFs;
uv in the file's units), data (nchannels, nstokes, nrows) complex128, sigma = weight^-1/2
where the weight is positive (0 elsewhere) and the mask weight > 0; with combine_stokes the
first two Stokes products are averaged, sigma = sqrt(s1^2 + s2^2)/2, masked unless both are
valid.
"""
from __future__ import annotations

import numpy as np

BLOCK = 2880

_TFORM = {"L": ("?", 1), "B": ("u1", 1), "I": (">i2", 2), "J": (">i4", 4), "K": (">i8", 8),
          "A": ("S1", 1), "E": (">f4", 4), "D": (">f8", 8), "C": (">c8", 8), "M": (">c16", 16)}
_BITPIX = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


def _value(s):
    s = s.strip()
    if s.startswith("'"):
        end = s.find("'", 1)
        while end != -1 and end + 1 < len(s) and s[end + 1] == "'":
            end = s.find("'", end + 2)
        return s[1:end].replace("''", "'").rstrip()
    v = s.split("/", 1)[0].strip()
    if v in ("T", "F"):
        return v == "T"
    try:
        return int(v)
    except ValueError:
        pass
    try:
        return float(v.replace("D", "E"))
    except ValueError:
        return v


def _header(buf, off):
    """(ordered dict of keyword -> value, offset after the header blocks)."""
    cards = {}
    while True:
        if off + BLOCK > len(buf):
            raise ValueError("truncated FITS header")
        blk = buf[off:off + BLOCK]
        off += BLOCK
        for i in range(36):
            card = blk[80 * i:80 * (i + 1)].decode("ascii", "replace")
            key = card[:8].strip()
            if key == "END":
                return cards, off
            if card[8:10] == "= " and key:
                cards[key] = _value(card[10:])


def read_hdus(path):
    """[(header, data bytes)] for every HDU of a FITS file."""
    with open(path, "rb") as f:
        buf = f.read()
    out, off = [], 0
    while off < len(buf):
        if not buf[off:off + 6].strip(b" \x00"):
            break
        h, off = _header(buf, off)
        naxis = h.get("NAXIS", 0)
        dims = [h.get(f"NAXIS{i}", 0) for i in range(1, naxis + 1)]
        if h.get("GROUPS") and naxis and dims[0] == 0:
            n = h.get("GCOUNT", 1) * (h.get("PCOUNT", 0) + int(np.prod(dims[1:])))
        else:
            n = (int(np.prod(dims)) + h.get("PCOUNT", 0)) * h.get("GCOUNT", 1) if dims else 0
            if h.get("XTENSION", "").startswith("BINTABLE"):
                n = dims[0] * dims[1] + h.get("PCOUNT", 0)
        nbytes = n * abs(h.get("BITPIX", 8)) // 8
        out.append((h, buf[off:off + nbytes]))
        off += (nbytes + BLOCK - 1) // BLOCK * BLOCK
    return out


def random_groups(h, data):
    """(parameters by name -> float64 array (GCOUNT,), data array (GCOUNT, NAXISn..NAXIS2))."""
    dt = np.dtype(_BITPIX[h["BITPIX"]])
    naxis = h["NAXIS"]
    shape = [h[f"NAXIS{i}"] for i in range(naxis, 1, -1)]
    pc, gc = h["PCOUNT"], h["GCOUNT"]
    arr = np.frombuffer(data, dtype=dt, count=gc * (pc + int(np.prod(shape)))).reshape(gc, -1)
    params = {}
    for i in range(1, pc + 1):
        name = str(h.get(f"PTYPE{i}", f"PARAM{i}")).strip().upper()
        v = arr[:, i - 1].astype(np.float64) * h.get(f"PSCAL{i}", 1.0) + h.get(f"PZERO{i}", 0.0)
        params[name] = params[name] + v if name in params else v
    vals = arr[:, pc:].astype(np.float64) * h.get("BSCALE", 1.0) + h.get("BZERO", 0.0)
    return params, vals.reshape([gc] + shape)


def bintable(h, data):
    """Columns of a binary table: name -> array (NAXIS2, repeat) (strings as bytes)."""
    nrows, rowlen = h["NAXIS2"], h["NAXIS1"]
    fields, off = [], 0
    for i in range(1, h["TFIELDS"] + 1):
        form = str(h[f"TFORM{i}"]).strip()
        k = 0
        while k < len(form) and form[k].isdigit():
            k += 1
        rep = int(form[:k]) if k else 1
        code = form[k]
        dt, size = _TFORM[code]
        fields.append((str(h.get(f"TTYPE{i}", f"COL{i}")).strip(), off, dt, rep))
        off += size * rep
    raw = np.frombuffer(data, dtype=np.uint8, count=nrows * rowlen).reshape(nrows, rowlen)
    cols = {}
    for name, o, dt, rep in fields:
        size = np.dtype(dt).itemsize
        cols[name] = raw[:, o:o + size * rep].copy().view(dt).reshape(nrows, rep)
    return cols


def load_uvfits(path, combine_stokes=False):
    """(VisibilitySpace, data (nch, nstokes, nrows) c128, sigma f64, mask bool), as
    lentils/common/data_util.py:5-76 returns them."""
    from .spaces import VisibilitySpace
    hdus = read_hdus(path)
    h, data = hdus[0]
    if not (h.get("GROUPS") and h.get("NAXIS1", -1) == 0):
        raise ValueError("not a random-groups uvfits file")
    axes = {}
    for ax in range(1, h["NAXIS"] + 1):
        nax = h[f"NAXIS{ax}"]
        if nax == 0:
            continue
        axes[str(h[f"CTYPE{ax}"]).strip()] = {k: h.get(f"{k}{ax}", 0.0) for k in
                                               ("CRVAL", "CDELT", "CRPIX", "CROTA")}
        axes[str(h[f"CTYPE{ax}"]).strip()]["NAXIS"] = nax
    params, vals = random_groups(h, data)
    nrows = h["GCOUNT"]
    nspw = axes["IF"]["NAXIS"]
    nchan = axes["FREQ"]["NAXIS"]
    ref_freq = axes["FREQ"]["CRVAL"]
    ref_ch = axes["FREQ"]["CRPIX"] - 1
    fq = next((bintable(hh, dd) for hh, dd in hdus[1:]
               if str(hh.get("EXTNAME", "")).strip() == "AIPS FQ"), None)
    if fq is None:
        raise ValueError("uvfits file without an 'AIPS FQ' table")
    chw = fq["CH WIDTH"].astype(np.float64).reshape(nspw)
    iff = fq["IF FREQ"].astype(np.float64).reshape(nspw, 1)
    channels = (np.multiply.outer(chw, np.arange(nchan) - ref_ch) + iff + ref_freq).flatten()
    nch = nchan * nspw

    def param(name):
        for k, v in params.items():
            if k == name or k.startswith(name + "-"):
                return v
        raise KeyError(name)

    uvw = np.array([param("UU"), param("VV"), param("WW")]).T.astype(np.float64, order="C")
    # (rows, DEC, RA, IF, FREQ, STOKES, COMPLEX) -> first RA/DEC pixel
    d = vals[:, 0, 0]
    vis = d[..., 0] + 1j * d[..., 1]
    w = d[..., 2]
    mask = w > 0.0
    sigma = np.zeros_like(w)
    sigma[mask] = w[mask] ** -0.5
    if combine_stokes:
        mask = np.all(mask, axis=-1)
        vis = 0.5 * (vis[..., 0] + vis[..., 1])
        srr, sll = sigma[..., 0], sigma[..., 1]
        sigma = np.zeros_like(srr)
        sigma[mask] = 0.5 * np.sqrt(srr[mask] ** 2 + sll[mask] ** 2)
        nst = 1
    else:
        vis, sigma, mask = vis[..., 0], sigma[..., 0], mask[..., 0]
        nst = 1
    space = VisibilitySpace(channels=channels, uvcoords=uvw)

    def order(a, dt):
        return np.ascontiguousarray(np.moveaxis(a.reshape(nrows, nch, nst), [0, 1, 2],
                                                [2, 0, 1]).astype(dt))
    return space, order(vis, np.complex128), order(sigma, np.float64), order(mask, np.bool_)


def write_uvfits(path, uvw, vis, weights, freq, ch_width, if_freq, date=None):
    """A minimal random-groups uvfits file (for tests and examples): uvw (nrows, 3) in the
    file's units, vis / weights (nrows, nif, nchan, nstokes), reference frequency `freq`,
    per-IF channel widths and frequency offsets; one RA/DEC pixel, an 'AIPS FQ' table."""
    vis = np.asarray(vis)
    weights = np.asarray(weights, dtype=np.float64)
    nrows, nif, nchan, nst = vis.shape

    def cards(items):
        s = ""
        for k, v in items:
            if isinstance(v, bool):
                vs = f"{'T' if v else 'F':>20}"
            elif isinstance(v, str):
                vs = f"'{v:<8}'"
            elif isinstance(v, int):
                vs = f"{v:>20d}"
            else:
                vs = f"{v:>20.12E}"
            s += f"{k:<8}= {vs}".ljust(80)
        s += "END".ljust(80)
        s += " " * ((-len(s)) % BLOCK)
        return s.encode("ascii")

    ptypes = ["UU", "VV", "WW", "DATE", "BASELINE"]
    hdr = [("SIMPLE", True), ("BITPIX", -32), ("NAXIS", 7), ("NAXIS1", 0), ("NAXIS2", 3),
           ("NAXIS3", nst), ("NAXIS4", nchan), ("NAXIS5", nif), ("NAXIS6", 1), ("NAXIS7", 1),
           ("EXTEND", True), ("GROUPS", True), ("PCOUNT", len(ptypes)), ("GCOUNT", nrows),
           ("BSCALE", 1.0), ("BZERO", 0.0)]
    for i, (ct, cv, cd) in enumerate((("COMPLEX", 1.0, 1.0), ("STOKES", -1.0, -1.0),
                                      ("FREQ", float(freq), float(ch_width[0])),
                                      ("IF", 1.0, 1.0), ("RA", 0.0, 1.0), ("DEC", 0.0, 1.0)),
                                     start=2):
        hdr += [(f"CTYPE{i}", ct), (f"CRVAL{i}", cv), (f"CDELT{i}", cd), (f"CRPIX{i}", 1.0),
                (f"CROTA{i}", 0.0)]
    for i, p in enumerate(ptypes, start=1):
        hdr += [(f"PTYPE{i}", p), (f"PSCAL{i}", 1.0), (f"PZERO{i}", 0.0)]
    par = np.zeros((nrows, len(ptypes)))
    par[:, :3] = uvw
    par[:, 3] = 2456222.5 if date is None else date
    par[:, 4] = 256 + 2
    arr = np.zeros((nrows, 1, 1, nif, nchan, nst, 3))
    arr[:, 0, 0, ..., 0] = vis.real
    arr[:, 0, 0, ..., 1] = vis.imag
    arr[:, 0, 0, ..., 2] = weights
    body = np.concatenate([par, arr.reshape(nrows, -1)], axis=1).astype(">f4").tobytes()
    body += b"\0" * ((-len(body)) % BLOCK)
    fq_cols = [("FRQSEL", "1J"), ("IF FREQ", f"{nif}D"), ("CH WIDTH", f"{nif}E"),
               ("TOTAL BANDWIDTH", f"{nif}E"), ("SIDEBAND", f"{nif}J")]
    rowlen = 4 + 8 * nif + 4 * nif + 4 * nif + 4 * nif
    th = [("XTENSION", "BINTABLE"), ("BITPIX", 8), ("NAXIS", 2), ("NAXIS1", rowlen),
          ("NAXIS2", 1), ("PCOUNT", 0), ("GCOUNT", 1), ("TFIELDS", len(fq_cols))]
    for i, (n, fm) in enumerate(fq_cols, start=1):
        th += [(f"TTYPE{i}", n), (f"TFORM{i}", fm)]
    th += [("EXTNAME", "AIPS FQ"), ("NO_IF", nif)]
    row = (np.array([1], ">i4").tobytes() + np.asarray(if_freq, ">f8").tobytes()
           + np.asarray(ch_width, ">f4").tobytes()
           + (np.asarray(ch_width, ">f4") * nchan).astype(">f4").tobytes()
           + np.ones(nif, ">i4").tobytes())
    row += b"\0" * ((-len(row)) % BLOCK)
    with open(path, "wb") as f:
        f.write(cards(hdr) + body + cards(th) + row)
