"""An independent decoder of uvfits files for the loader's parity test.

It reads the FITS random-groups standard directly with numpy structured dtypes -- a second
implementation that shares no code with lentils_gb300/uvfits.py -- and applies the reference
loader's rules (lentils/common/data_util.py:5-76) to what it decodes:

  * the primary header's cards are split with a regular expression; a group is one record of
    PCOUNT parameters followed by the NAXIS2 x ... x NAXISn array, both big-endian of BITPIX;
  * uvw = the parameters named UU, VV, WW (each times PSCALn plus PZEROn, parameters of one
    name summed, as astropy's GroupData field access does);
  * the array's last axes are (..., IF, FREQ, STOKES, COMPLEX) in C order; data = re + i im,
    weights = the third COMPLEX element, times BSCALE plus BZERO;
  * the 'AIPS FQ' binary table gives 'IF FREQ' and 'CH WIDTH' per IF; channel frequencies are
    CH WIDTH x (channel - (CRPIX - 1)) + IF FREQ + CRVAL of the FREQ axis, IF-major.
"""
import re

import numpy as np

_CARD = re.compile(r"^([A-Z0-9_-]{1,8})\s*=\s*('(?:[^']|'')*'|[^/]*)")
_NP = {8: "u1", 16: "i2", 32: "i4", 64: "i8", -32: "f4", -64: "f8"}
_BIN = {"E": "f4", "D": "f8", "J": "i4", "I": "i2", "K": "i8", "B": "u1", "A": "S"}


def _parse(value):
    value = value.strip()
    if value.startswith("'"):
        return value[1:-1].replace("''", "'").rstrip()
    if value in ("T", "F"):
        return value == "T"
    for conv in (int, float):
        try:
            return conv(value.replace("D", "E") if conv is float else value)
        except ValueError:
            continue
    return value


def _headers(raw):
    """Yield (cards, data offset) for each HDU; a repeated keyword keeps its first value."""
    pos = 0
    while pos + 2880 <= len(raw) and raw[pos:pos + 8].strip():
        cards, done = {}, False
        while not done:
            block = raw[pos:pos + 2880].decode("ascii")
            pos += 2880
            for k in range(0, 2880, 80):
                line = block[k:k + 80]
                if line.startswith("END") and not line[3:].strip():
                    done = True
                    break
                m = _CARD.match(line)
                if m:
                    cards.setdefault(m.group(1), _parse(m.group(2)))
        yield cards, pos
        naxes = [cards.get(f"NAXIS{i}", 0) for i in range(1, cards.get("NAXIS", 0) + 1)]
        if cards.get("GROUPS"):
            nbytes = cards["GCOUNT"] * (cards["PCOUNT"] + int(np.prod(naxes[1:])))
        else:
            nbytes = int(np.prod(naxes)) + cards.get("PCOUNT", 0) if naxes else 0
        nbytes *= abs(cards.get("BITPIX", 8)) // 8
        pos += -(-nbytes // 2880) * 2880


def decode(path, combine_stokes=False):
    """(uvw, channels, data, sigma, mask) with the reference loader's shapes:
    data / sigma / mask are (nchannels, nstokes, nrows)."""
    raw = open(path, "rb").read()
    hdus = list(_headers(raw))
    prim, off = hdus[0]
    naxis = prim["NAXIS"]
    shape = tuple(prim[f"NAXIS{i}"] for i in range(naxis, 1, -1))  # C order, COMPLEX last
    vt = ">" + _NP[prim["BITPIX"]]
    rec = np.dtype([("p", vt, (prim["PCOUNT"],)), ("a", vt, shape)])
    groups = np.frombuffer(raw, rec, prim["GCOUNT"], off)
    params = groups["p"].astype(np.float64)
    names = [prim[f"PTYPE{i}"].strip() for i in range(1, prim["PCOUNT"] + 1)]

    def par(name):
        cols = [i for i, nm in enumerate(names) if nm == name]
        return sum(params[:, i] * prim.get(f"PSCAL{i + 1}", 1.0) + prim.get(f"PZERO{i + 1}", 0.0)
                   for i in cols)
    uvw = np.stack([par("UU"), par("VV"), par("WW")], axis=1)
    arr = groups["a"].astype(np.float64) * prim.get("BSCALE", 1.0) + prim.get("BZERO", 0.0)
    ctype = {prim[f"CTYPE{i}"].strip(): i for i in range(2, naxis + 1)}
    # collapse every axis but IF, FREQ, STOKES, COMPLEX (RA, DEC have length 1)
    nif, nfreq = prim[f"NAXIS{ctype['IF']}"], prim[f"NAXIS{ctype['FREQ']}"]
    nst = prim[f"NAXIS{ctype['STOKES']}"]
    arr = arr.reshape(arr.shape[0], nif, nfreq, nst, 3)
    vis = arr[..., 0] + 1j * arr[..., 1]
    wts = arr[..., 2]
    # AIPS FQ table
    fq, foff = next((h, o) for h, o in hdus[1:] if h.get("EXTNAME") == "AIPS FQ")
    cols = []
    for i in range(1, fq["TFIELDS"] + 1):
        form = re.match(r"(\d*)([A-Z])", fq[f"TFORM{i}"].strip())
        rep = int(form.group(1) or 1)
        code = _BIN[form.group(2)]
        dt = (f"S{rep}",) if code == "S" else (">" + code, (rep,)) if rep > 1 else (">" + code,)
        cols.append((fq[f"TTYPE{i}"].strip(), *dt))
    table = np.frombuffer(raw, np.dtype(cols), fq["NAXIS2"], foff)
    fi = ctype["FREQ"]
    chans = (np.asarray(table["CH WIDTH"], np.float64).reshape(nif, 1)
             * (np.arange(nfreq) - (prim[f"CRPIX{fi}"] - 1))
             + np.asarray(table["IF FREQ"], np.float64).reshape(nif, 1)
             + prim[f"CRVAL{fi}"]).reshape(-1)
    mask = wts > 0
    sig = np.zeros_like(wts)
    sig[mask] = wts[mask] ** -0.5
    if combine_stokes:
        m = mask[..., 0] & mask[..., 1]
        vis = 0.5 * (vis[..., 0] + vis[..., 1])
        s2 = np.zeros(m.shape)
        s2[m] = 0.5 * np.sqrt(sig[..., 0][m] ** 2 + sig[..., 1][m] ** 2)
        sig, mask = s2, m
    else:
        vis, sig, mask = vis[..., 0], sig[..., 0], mask[..., 0]
    nrows = vis.shape[0]
    order = lambda a: np.transpose(a.reshape(nrows, nif * nfreq, 1), (1, 2, 0))  # noqa: E731
    return uvw, chans, order(vis), order(sig), order(mask)
