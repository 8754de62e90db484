"""Minimal FITS reader/writer for the correlation inputs and outputs.

picca reads and writes FITS through the third-party ``fitsio`` package
(``py/picca/io.py:19``, ``py/picca/bin/picca_cf.py:14``). That package is not
part of this project's environment, so this module implements the subset of
the FITS standard (Pence et al. 2010, A&A 524, A42) that the hot path needs:

* reading gzip-compressed or plain files made of a primary HDU followed by
  BINTABLE and IMAGE extensions (fixed-width columns of type L, B, I, J, K,
  E, D and A, scalar or vector);
* writing a primary HDU plus BINTABLE extensions with header records, which
  is what ``picca_cf.py`` / ``picca_xcf.py`` produce (``ATTRI`` and ``COR``).

The interface is deliberately small: :func:`read_hdus` returns a list of
:class:`HDU` objects and :class:`FITS` gives the ``hdul["NAME"]`` /
``hdu["COLUMN"][:]`` / ``hdu.read_header()`` access pattern that the delta
readers in ``py/picca/data.py:376-620`` use.
"""

import gzip
import io
import os

import numpy as np

BLOCK = 2880
CARD = 80

_BINTABLE_TYPES = {
    "L": ("i1", 1),
    "B": ("u1", 1),
    "I": (">i2", 2),
    "J": (">i4", 4),
    "K": (">i8", 8),
    "E": (">f4", 4),
    "D": (">f8", 8),
    "A": ("S", 1),
}

_IMAGE_TYPES = {8: "u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


class FITSError(RuntimeError):
    """Raised when a file cannot be parsed as FITS."""


class Header(dict):
    """Ordered keyword dictionary that also keeps the raw records."""

    def __init__(self):
        super().__init__()
        self.record_list = []

    def records(self):
        """Return the header records as dictionaries (name, value, comment)."""
        return list(self.record_list)


def _parse_value(text):
    text = text.strip()
    if not text:
        return None
    if text.startswith("'"):
        # string value, '' escapes a quote
        out = []
        i = 1
        while i < len(text):
            if text[i] == "'":
                if i + 1 < len(text) and text[i + 1] == "'":
                    out.append("'")
                    i += 2
                    continue
                break
            out.append(text[i])
            i += 1
        return "".join(out).rstrip()
    if text == "T":
        return True
    if text == "F":
        return False
    try:
        return int(text)
    except ValueError:
        pass
    try:
        return float(text.replace("D", "E"))
    except ValueError:
        return text


def _split_value_comment(text):
    """Split the value field of a card into (value, comment)."""
    text = text.rstrip()
    if text.lstrip().startswith("'"):
        start = text.index("'")
        i = start + 1
        while i < len(text):
            if text[i] == "'":
                if i + 1 < len(text) and text[i + 1] == "'":
                    i += 2
                    continue
                break
            i += 1
        value = text[: i + 1]
        rest = text[i + 1:]
        comment = rest.split("/", 1)[1].strip() if "/" in rest else ""
        return value, comment
    if "/" in text:
        value, comment = text.split("/", 1)
        return value, comment.strip()
    return text, ""


class HDU:
    """One header-data unit: ``kind`` is 'primary', 'image' or 'bintable'."""

    def __init__(self, header, kind, data):
        self.header = header
        self.kind = kind
        self._data = data

    # fitsio-like accessors -------------------------------------------------
    def read_header(self):
        return self.header

    def get_colnames(self):
        if self.kind != "bintable":
            return []
        return list(self._data.dtype.names)

    def get_nrows(self):
        if self.kind != "bintable":
            raise FITSError("not a table")
        return len(self._data)

    def read(self):
        if self.kind == "bintable":
            return self._data
        return self._data

    def __getitem__(self, key):
        if self.kind == "bintable":
            names = {n.upper(): n for n in self._data.dtype.names}
            col = self._data[names[key.upper()]]
            return _native(col)
        return _native(self._data)[key]

    @property
    def name(self):
        return str(self.header.get("EXTNAME", "")).strip()


def _native(arr):
    """Convert a big-endian numpy array to native byte order."""
    if arr.dtype.kind in "SU":
        return np.char.rstrip(arr.astype("U"))
    if arr.dtype.byteorder not in ("=", "|"):
        return arr.astype(arr.dtype.newbyteorder("="))
    return np.array(arr)


def _read_raw(path):
    with open(path, "rb") as handle:
        raw = handle.read()
    if raw[:2] == b"\x1f\x8b":
        raw = gzip.decompress(raw)
    return raw


def _parse_header(raw, pos):
    header = Header()
    while True:
        if pos + BLOCK > len(raw):
            raise FITSError("truncated header")
        block = raw[pos:pos + BLOCK]
        pos += BLOCK
        done = False
        for i in range(BLOCK // CARD):
            card = block[i * CARD:(i + 1) * CARD].decode("ascii", "replace")
            name = card[:8].strip()
            if name == "END":
                done = True
                break
            if name == "HIERARCH" and "=" in card[9:]:
                # ESO HIERARCH convention (cfitsio writes keywords longer than
                # eight characters this way): "HIERARCH NAME = value / comment"
                key, rest = card[9:].split("=", 1)
                value_text, comment = _split_value_comment(rest)
                value = _parse_value(value_text)
                name = key.strip()
                header[name] = value
                header.record_list.append({"name": name, "value": value, "comment": comment})
            elif card[8:10] == "= ":
                value_text, comment = _split_value_comment(card[10:])
                value = _parse_value(value_text)
                header[name] = value
                header.record_list.append(
                    {"name": name, "value": value, "comment": comment})
            elif name:
                header.record_list.append(
                    {"name": name, "value": card[8:].rstrip(), "comment": ""})
        if done:
            break
    return header, pos


def _bintable_dtype(header):
    fields = []
    for index in range(1, header["TFIELDS"] + 1):
        name = str(header.get(f"TTYPE{index}", f"COL{index}")).strip()
        form = str(header[f"TFORM{index}"]).strip()
        digits = ""
        k = 0
        while k < len(form) and form[k].isdigit():
            digits += form[k]
            k += 1
        repeat = int(digits) if digits else 1
        code = form[k]
        if code not in _BINTABLE_TYPES:
            raise FITSError(f"unsupported TFORM {form}")
        base, _ = _BINTABLE_TYPES[code]
        if code == "A":
            fields.append((name, f"S{repeat}"))
        elif repeat == 1:
            fields.append((name, base))
        else:
            fields.append((name, base, (repeat,)))
    return np.dtype(fields)


def hdu_headers(raw):
    """The header of every HDU of an uncompressed FITS byte string, without
    reading any data."""
    pos = 0
    headers = []
    while pos < len(raw) and raw[pos:pos + BLOCK].strip(b"\x00 "):
        header, pos = _parse_header(raw, pos)
        naxis = header["NAXIS"]
        nbytes = 0
        if naxis > 0:
            nbytes = abs(header["BITPIX"]) // 8
            for i in range(1, naxis + 1):
                nbytes *= header[f"NAXIS{i}"]
        nbytes += header.get("PCOUNT", 0) or 0
        headers.append(header)
        pos += (nbytes + BLOCK - 1) // BLOCK * BLOCK
    return headers


def read_hdus(path):
    """Read every HDU of a (possibly gzip-compressed) FITS file."""
    raw = _read_raw(path)
    pos = 0
    hdus = []
    while pos < len(raw):
        if not raw[pos:pos + BLOCK].strip(b"\x00 "):
            break
        header, pos = _parse_header(raw, pos)
        bitpix = header["BITPIX"]
        naxis = header["NAXIS"]
        dims = [header[f"NAXIS{i}"] for i in range(1, naxis + 1)]
        nbytes = 0
        if naxis > 0:
            nbytes = abs(bitpix) // 8
            for dim in dims:
                nbytes *= dim
        nbytes += header.get("PCOUNT", 0) or 0
        chunk = raw[pos:pos + nbytes]
        xtension = str(header.get("XTENSION", "")).strip()
        if xtension == "BINTABLE":
            dtype = _bintable_dtype(header)
            if dtype.itemsize != dims[0]:
                raise FITSError("row width mismatch")
            data = np.frombuffer(chunk, dtype=dtype, count=dims[1])
            if dtype.names:
                for index, fname in enumerate(dtype.names, start=1):
                    form = str(header[f"TFORM{index}"]).strip()
                    if form.endswith("L"):
                        pass
            hdus.append(HDU(header, "bintable", data))
        elif naxis == 0:
            hdus.append(HDU(header, "primary" if not hdus else "image", None))
        else:
            dtype = np.dtype(_IMAGE_TYPES[bitpix])
            count = int(np.prod(dims))
            data = np.frombuffer(chunk[:count * dtype.itemsize], dtype=dtype)
            data = data.reshape(tuple(reversed(dims)))
            scale = header.get("BSCALE", 1)
            zero = header.get("BZERO", 0)
            if scale != 1 or zero != 0:
                data = data.astype(float) * scale + zero
            hdus.append(HDU(header, "primary" if not hdus else "image", data))
        pos += (nbytes + BLOCK - 1) // BLOCK * BLOCK
    return hdus


class FITS:
    """Read-only container with ``fitsio.FITS``-like indexing."""

    def __init__(self, path):
        self.path = path
        self.hdus = read_hdus(path)

    def __len__(self):
        return len(self.hdus)

    def __iter__(self):
        return iter(self.hdus)

    def __contains__(self, name):
        return any(h.name == name for h in self.hdus)

    def __getitem__(self, key):
        if isinstance(key, slice):
            return self.hdus[key]
        if isinstance(key, int):
            return self.hdus[key]
        for hdu in self.hdus:
            if hdu.name == key:
                return hdu
        raise KeyError(key)

    def close(self):
        self.hdus = []

    def __enter__(self):
        return self

    def __exit__(self, *args):
        self.close()


# --------------------------------------------------------------------------
# writing
# --------------------------------------------------------------------------
def _format_value(value):
    if isinstance(value, (bool, np.bool_)):
        return f"{'T' if value else 'F':>20}"
    if value is None:
        return " " * 20
    if isinstance(value, (int, np.integer)):
        return f"{int(value):>20d}"
    if isinstance(value, (float, np.floating)):
        text = repr(float(value)).upper()
        if "E" not in text and "." not in text and "INF" not in text and "NAN" not in text:
            text += ".0"
        return f"{text:>20}"
    text = str(value).replace("'", "''")
    text = f"'{text:<8}'"
    return f"{text:<20}"


def _card(name, value=None, comment=""):
    if name in ("COMMENT", "HISTORY", ""):
        card = f"{name:<8}{str(value or '')}"
    elif len(name) > 8:
        card = f"HIERARCH {name} = {_format_value(value).strip()}"
        if len(card) > CARD:
            raise ValueError(f"HIERARCH card for {name!r} needs {len(card)} characters "
                             f"(a card holds {CARD})")
        if comment and len(card) + 3 + len(comment) <= CARD:
            card += f" / {comment}"
        return card.ljust(CARD)
    else:
        card = f"{name:<8}= {_format_value(value)}"
        if comment:
            card += f" / {comment}"
    return card[:CARD].ljust(CARD)


def _header_bytes(cards):
    cards = list(cards) + ["END".ljust(CARD)]
    text = "".join(cards)
    pad = (-len(text)) % BLOCK
    return (text + " " * pad).encode("ascii")


def _pad_data(buf):
    pad = (-len(buf)) % BLOCK
    return buf + b"\x00" * pad


def _column_spec(values):
    arr = np.asarray(values)
    if arr.dtype.kind == "b":
        return "L", arr.astype("i1") * ord("T") + (~arr).astype("i1") * ord("F"), 1
    if arr.dtype.kind in "iu":
        if arr.dtype.itemsize <= 2 and arr.dtype.kind == "i":
            return "I", arr.astype(">i2"), 2
        if arr.dtype.itemsize <= 4 and arr.dtype.kind == "i":
            return "J", arr.astype(">i4"), 4
        return "K", arr.astype(">i8"), 8
    if arr.dtype.kind == "f":
        if arr.dtype.itemsize == 4:
            return "E", arr.astype(">f4"), 4
        return "D", arr.astype(">f8"), 8
    if arr.dtype.kind in "SU":
        width = max(1, int(arr.astype("S").dtype.itemsize))
        return "A", arr.astype(f"S{width}"), width
    raise FITSError(f"cannot write column of dtype {arr.dtype}")


def _primary_bytes(records=None):
    return _header_bytes([
        _card("SIMPLE", True, "file does conform to FITS standard"),
        _card("BITPIX", 8, "number of bits per data pixel"),
        _card("NAXIS", 0, "number of data axes"),
        _card("EXTEND", True, "FITS dataset may contain extensions"),
    ] + [_card(r["name"], r["value"], r.get("comment", "")) for r in (records or [])])


def _table_bytes(table):
    columns = table["columns"]
    names = table["names"]
    units = table.get("units") or [""] * len(names)
    comments = table.get("comments") or [""] * len(names)
    nrows = len(np.asarray(columns[0]))
    specs = []
    row_fields = []
    for col, name in zip(columns, names):
        arr = np.asarray(col)
        if arr.shape[0] != nrows:
            raise FITSError("columns must share their first dimension")
        code, conv, width = _column_spec(arr)
        repeat = int(np.prod(arr.shape[1:])) if arr.ndim > 1 else 1
        if code == "A":
            tform = f"{width}A"
            field_dtype = conv.dtype
        else:
            tform = f"{repeat}{code}" if repeat != 1 else code
            field_dtype = conv.dtype if repeat == 1 else (conv.dtype, (repeat,))
        specs.append((name, tform))
        row_fields.append((name, conv.reshape(nrows, -1) if repeat != 1 else conv,
                           field_dtype))
    dtype = np.dtype([(n, d) for n, _, d in row_fields])
    rec = np.zeros(nrows, dtype=dtype)
    for name, conv, _ in row_fields:
        rec[name] = conv
    cards = [
        _card("XTENSION", "BINTABLE", "binary table extension"),
        _card("BITPIX", 8, "8-bit bytes"),
        _card("NAXIS", 2, "2-dimensional binary table"),
        _card("NAXIS1", dtype.itemsize, "width of table in bytes"),
        _card("NAXIS2", nrows, "number of rows in table"),
        _card("PCOUNT", 0, "size of special data area"),
        _card("GCOUNT", 1, "one data group (required keyword)"),
        _card("TFIELDS", len(specs), "number of fields in each row"),
    ]
    for index, ((name, tform), unit, comment) in enumerate(
            zip(specs, units, comments), start=1):
        cards.append(_card(f"TTYPE{index}", name, comment or f"label for field {index}"))
        cards.append(_card(f"TFORM{index}", tform, "data format of field"))
        if unit:
            cards.append(_card(f"TUNIT{index}", unit, "physical unit of field"))
    if table.get("extname"):
        cards.append(_card("EXTNAME", table["extname"], "name of this binary table extension"))
    for record in table.get("header") or []:
        cards.append(_card(record["name"], record["value"], record.get("comment", "")))
    return _header_bytes(cards) + _pad_data(rec.tobytes())


def _image_bytes(extname, arr, records):
    arr = np.asarray(arr)
    if arr.dtype.kind == "f":
        bitpix, data = -64, arr.astype(">f8")
    else:
        bitpix, data = 64, arr.astype(">i8")
    cards = [
        _card("XTENSION", "IMAGE", "Image extension"),
        _card("BITPIX", bitpix, "data type"),
        _card("NAXIS", arr.ndim, "number of axes"),
    ]
    for axis, dim in enumerate(reversed(arr.shape), start=1):
        cards.append(_card(f"NAXIS{axis}", dim))
    cards += [_card("PCOUNT", 0), _card("GCOUNT", 1), _card("EXTNAME", extname)]
    for record in records or []:
        cards.append(_card(record["name"], record["value"], record.get("comment", "")))
    return _header_bytes(cards) + _pad_data(data.tobytes())


def _write_payload(path, payload):
    if str(path).endswith(".gz"):
        payload = gzip.compress(payload, compresslevel=4)
    with open(path, "wb") as handle:
        handle.write(payload)


def write_fits(path, tables, clobber=True):
    """Write a primary HDU followed by one BINTABLE per entry of ``tables``.

    Each entry is a dict with keys ``columns`` (list of arrays), ``names``,
    optional ``units``, ``comments``, ``header`` (list of
    ``{"name","value","comment"}`` records) and ``extname``. Arrays of shape
    (nrows, k) become vector columns ``kD``/``kK``. A ``.gz`` suffix gzips the
    output, as ``fitsio`` does.
    """
    if os.path.exists(path) and not clobber:
        raise FITSError(f"{path} exists")
    out = io.BytesIO()
    out.write(_primary_bytes())
    for table in tables:
        out.write(_table_bytes(table))
    _write_payload(path, out.getvalue())


def write_hdus(path, hdus, primary_header=None):
    """Write a primary HDU and a mix of extensions: each entry of ``hdus`` is
    ``("image", extname, array, header records)`` or ``("table", table)``
    with ``table`` as for :func:`write_fits`."""
    out = io.BytesIO()
    out.write(_primary_bytes(primary_header))
    for entry in hdus:
        if entry[0] == "image":
            out.write(_image_bytes(*entry[1:]))
        else:
            out.write(_table_bytes(entry[1]))
    _write_payload(path, out.getvalue())


def write_image_hdus(path, images, primary_header=None):
    """Write a primary HDU plus IMAGE extensions (used by fixture writers).

    ``images`` is a list of (extname, array, header records). Arrays are
    written big-endian as float64 (BITPIX -64) or int64 (BITPIX 64).
    """
    write_hdus(path, [("image",) + tuple(entry) for entry in images], primary_header)
