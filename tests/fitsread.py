"""A small FITS reader for the tests (primary header keys and binary tables
of FP64 columns), independent of the C++ writer it checks."""
from __future__ import annotations

import numpy as np

BLOCK = 2880


def _cards(buf: bytes, off: int):
    cards = []
    while True:
        card = buf[off:off + 80].decode("ascii")
        off += 80
        if card.startswith("END") and card[3:].strip() == "":
            break
        cards.append(card)
    return cards, (off + BLOCK - 1) // BLOCK * BLOCK


def _parse(card: str):
    if card.startswith("HIERARCH "):
        name, _, rest = card[9:].partition("=")
    elif card[8:10] == "= ":
        name, rest = card[:8], card[10:]
    else:
        return None
    rest = rest.strip()
    if rest.startswith("'"):
        value = rest[1:rest.index("'", 1)].rstrip()
    else:
        value = rest.split("/")[0].strip()
        if value in ("T", "F"):
            value = value == "T"
        else:
            try:
                value = int(value)
            except ValueError:
                value = float(value.replace("D", "E"))
    return name.strip().upper(), value


def read_fits(path: str):
    """(primary keys, {EXTNAME: {column name: array [rows, repeat]}})."""
    buf = open(path, "rb").read()
    assert len(buf) % BLOCK == 0, "FITS files are whole 2880-byte blocks"
    off = 0
    primary = None
    tables = {}
    while off < len(buf):
        cards, data_off = _cards(buf, off)
        keys = dict(kv for kv in map(_parse, cards) if kv)
        if primary is None:
            assert keys["SIMPLE"] is True
            primary = keys
            size = 0 if keys["NAXIS"] == 0 else None
            assert size == 0
        else:
            assert keys["XTENSION"] == "BINTABLE" and keys["BITPIX"] == 8 and keys["NAXIS"] == 2
            w, rows = keys["NAXIS1"], keys["NAXIS2"]
            size = w * rows + keys["PCOUNT"]
            cols = {}
            o = 0
            raw = np.frombuffer(buf, dtype=np.uint8, count=w * rows, offset=data_off).reshape(rows, w)
            for c in range(1, keys["TFIELDS"] + 1):
                form = keys[f"TFORM{c}"]
                assert form.endswith("D")
                rep = int(form[:-1] or 1)
                cols[keys[f"TTYPE{c}"]] = raw[:, o:o + 8 * rep].copy().view(">f8").astype(np.float64)
                o += 8 * rep
            assert o == w
            tables[keys["EXTNAME"]] = cols
        off = data_off + (size + BLOCK - 1) // BLOCK * BLOCK
    return primary, tables
