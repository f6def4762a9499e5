"""Test infrastructure only (the oracle of the recovered-file list): a plain-Python restatement of
gpuzip's TarReader, the walk over a rescued tar stream (output bytes and their per-byte mask) that
decides which files are intact, suspect, inferred or partial (src/rescue.rs:374-829), followed by
the two rules that turn intact files into unverified ones (src/main.rs:546-558).

The reference is Rust and is not built here, so this restatement is pinned by reading those lines
and by the reference's own test of the reader (src/rescue.rs:853-898: a damaged tar read in
chunks reads as one read whole, with partial, suspect, inferred and skipped entries; an undamaged
one reads every file intact), restated in tests/test_tar_oracle.py. The reader runs here with no
output folder, as `untar(data, mask, None, false)` does (src/rescue.rs:406-411): nothing is
written, so links, folders and failures do not arise.
"""

UNKNOWN, EXACT, SUSPECT, INFERRED = 0, 1, 2, 3
MAX_META = 64 << 20  # src/rescue.rs:415


def rust_usize(b):
    """bytes b read as Rust's str::parse::<usize> (or ::<u64>) reads them: one optional '+', then
    one or more ASCII digits, below 2**64; None otherwise (Python's int() would also take spaces,
    underscores and a '-')."""
    s = b[1:] if b[:1] == b"+" else b
    if not s or any(c < 0x30 or c > 0x39 for c in s):
        return None
    v = int(s)
    return v if v < 1 << 64 else None


def octal(field):
    """A tar number field (src/rescue.rs:374-384): GNU base-256, or octal digits up to NUL or
    space; None when the digits do not parse."""
    if field and field[0] & 0x80:
        v = 0
        for b in field[1:]:
            v = (v << 8 | b) & 0xFFFFFFFFFFFFFFFF
        return v
    s = bytearray()
    for b in field:
        if b == 0 or b == 0x20:
            break
        s.append(b)
    if not s:
        return 0
    ws = set(range(0x09, 0x0E)) | {0x20, 0x85, 0xA0}  # Rust's trim, on Latin-1 characters
    a, e = 0, len(s)
    while a < e and s[a] in ws:
        a += 1
    while e > a and s[e - 1] in ws:
        e -= 1
    if a < e and s[a] == ord("+"):
        a += 1
    t = bytes(s[a:e])
    if not t or any(c not in b"01234567" for c in t):
        return None
    v = int(t, 8)
    return v if v < (1 << 64) else None


def header_valid(h):
    """The header checksum, as an unsigned or a signed byte sum (src/rescue.rs:386-395)."""
    want = octal(h[148:156])
    if want is None:
        return False
    unsigned = sum(h[:148]) + 8 * 0x20 + sum(h[156:512])
    signed = sum(b - 256 if b >= 128 else b for b in h[:148]) + 8 * 0x20 + sum(b - 256 if b >= 128 else b for b in h[156:512])
    return want == unsigned or (want if want < (1 << 63) else want - (1 << 64)) == signed


def field_str(f):
    """Bytes up to the first NUL, as text (src/rescue.rs:397-400)."""
    end = f.find(b"\0")
    return bytes(f if end < 0 else f[:end]).decode("utf-8", "replace")


def untar(data, mask, crc_check=-1, damaged=0, hidden_damage=0):
    """The outcome of reading the rescued tar `data` (with `mask`): a dict of intact (count),
    suspect, inferred, partial (names), skipped [(offset, bytes)], repaired (count), bytes (file
    bytes read) and unverified (count), the last after src/main.rs:546-558's rules."""
    total = len(data)
    o = {"intact": 0, "suspect": [], "inferred": [], "partial": [], "skipped": [], "repaired": 0, "bytes": 0,
         "unverified": 0}
    pos = 0
    long_name = pax_path = pax_size = long_link = pax_link = None
    last_valid = None
    prev_file = None  # (name, status, where the next header must be)

    def entry_done(body, cut, nxt):
        nonlocal prev_file, long_name, long_link, pax_path, pax_size, pax_link
        kind = body[0]
        if kind == "file":  # src/rescue.rs:769-800
            _, name, unknown, suspect, inferred, repaired = body
            status = 2 if (cut or unknown) else 1 if (repaired or suspect) else 3 if inferred else 0
            prev_file = (name, status, nxt)
            if status == 0:
                o["intact"] += 1
            elif status == 1:
                o["suspect"].append(name)
            elif status == 3:
                o["inferred"].append(name)
            else:
                o["partial"].append(name)
        elif kind == "meta":
            _, typeflag, buf = body
            if typeflag == ord("L"):
                long_name = field_str(buf)
            elif typeflag == ord("K"):
                long_link = field_str(buf)
            else:  # pax records "<len> key=value\n" (src/rescue.rs:804-825)
                p = 0
                while p < len(buf):
                    rec = buf[p:]
                    sp = rec.find(b" ")
                    if sp < 0:
                        break
                    n = rust_usize(bytes(rec[:sp]))
                    if n is None or n <= 0 or p + n > len(buf):
                        break
                    kv = buf[p + sp + 1:p + n - 1]
                    eq = kv.find(b"=")
                    if eq >= 0:
                        k, v = bytes(kv[:eq]), bytes(kv[eq + 1:]).decode("utf-8", "replace")
                        if k == b"path":
                            pax_path = v
                        elif k == b"linkpath":
                            pax_link = v
                        elif k == b"size":
                            pax_size = rust_usize(v.encode("utf-8", "surrogateescape"))
                    p += n

    while True:
        # ---- a header at pos (src/rescue.rs:646-763)
        if pos + 512 > total:
            break
        raw = bytes(data[pos:pos + 512])
        hmask = bytes(mask[pos:pos + 512])
        hbuf = bytearray(raw)
        repaired = False
        if not header_valid(hbuf) and UNKNOWN in hmask and last_valid is not None:
            for i in range(512):
                if hmask[i] == UNKNOWN:
                    hbuf[i] = last_valid[i]
            repaired = header_valid(hbuf)
        if raw.count(0) == 512:
            if hmask.count(EXACT) == 512:
                break  # the end-of-archive blocks
            valid = False
        else:
            valid = header_valid(hbuf)
        if valid:
            h = bytes(hbuf)
            last_valid = h
            if repaired:
                o["repaired"] += 1
            typeflag = h[156]
            prev_file = None
            size = pax_size if pax_size is not None else octal(h[124:136])
            pax_size = None
            if size is None:
                size = 0
            data_start = pos + 512
            end = min(data_start + size, (1 << 64) - 1)
            nxt = min(data_start + (size + 511) // 512 * 512, (1 << 64) - 1)
            if pax_path is not None:
                name, pax_path = pax_path, None
            elif long_name is not None:
                name, long_name = long_name, None
            else:
                base = field_str(h[0:100])
                prefix = field_str(h[345:500]) if h[257:262] == b"ustar" else ""
                name = f"{prefix}/{base}" if prefix else base
            name = name.replace("\\", "/")
            # the link target the header takes (nothing is made here): pax's, else GNU's
            if pax_link is not None:
                pax_link = None
            else:
                long_link = None
            if typeflag in (ord("L"), ord("K"), ord("x")):
                body = ["meta", typeflag, bytearray()]
            elif typeflag in (ord("0"), 0, ord("7")):
                body = ["file", name, False, False, False, repaired]
            else:
                body = ["skip"]
            # ---- its data (src/rescue.rs:574-608, read whole: eof)
            upto = min(end, total)
            if upto > data_start:
                m = bytes(mask[data_start:upto])
                if body[0] == "file":
                    body[2] = body[2] or UNKNOWN in m
                    body[3] = body[3] or SUSPECT in m
                    body[4] = body[4] or INFERRED in m
                    o["bytes"] += upto - data_start
                elif body[0] == "meta":
                    body[2] += bytes(data[data_start:upto])[:MAX_META]
            entry_done(body, upto < end, nxt)
            pos = nxt
            continue
        # ---- not a header: the file before it is suspect when this is where its next header
        # had to be and the bytes here are exact (src/rescue.rs:741-761)
        if prev_file is not None:
            name, status, at = prev_file
            if at == pos and all(m in (EXACT, INFERRED) for m in hmask):
                if status == 0:
                    o["intact"] -= 1
                    o["suspect"].append(name)
                elif status == 3:
                    o["inferred"] = [x for x in o["inferred"] if x != name]
                    o["suspect"].append(name)
        prev_file = None
        # ---- search byte by byte for the next header with a ustar magic (src/rescue.rs:610-633)
        start, q = pos, pos + 1
        found = None
        while q + 512 <= total:
            h = bytes(data[q:q + 512])
            if h[257:262] == b"ustar" and header_valid(h):
                found = q
                break
            q += 1
        if found is None:
            o["skipped"].append((start, total - start))
            break
        o["skipped"].append((start, found - start))
        pos = found
    # src/main.rs:546-558
    if crc_check == 0 and damaged == 0:
        o["unverified"] = o["intact"]
        o["intact"] = 0
    if hidden_damage:
        o["unverified"] += o["intact"]
        o["intact"] = 0
    return o
