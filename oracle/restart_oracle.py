"""Restatement of the reference's RESTART file layout, for the tests.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports or calls this file;
``tests/test_restart.py`` uses it as the checker of the library's
``gbcp_restart_write`` / ``gbcp_restart_read``: files written here are read by
the library and files written by the library are read here.

Parity unpinned: the reference ships no RESTART file and cannot be built here,
so the layout is restated from its source only:

* Fortran unformatted sequential records: 4-byte length before and after the
  data (gfortran); STREAM files (" STREAM" in the header) carry no frames.
* wv30_utils.mod.F90:235-470 ......... section 1 header string (80 chars),
  sections 2-8: (irecord, fpos) then irecord records; wv30_utils.mod.F90:
  1215-1260 ........................... sections 39-98 empty, 99 last.
* wfnio_utils.mod.F90:52-233 ......... section 9 (type 1): irecord = -(2n+3),
  pos = -1, (iwfntype), (n, ngwks, icompr, scale), (tlsd, nsup, nsdown), then
  per state wr30wfn_utils.mod.F90:460-564: (nx), (2 nx 32-bit words).
* compress.F90:1-130, 336-430 ......... icompr 1: FP64 as is; icompr 2, 4, 8:
  nb = 64/icompr bits, NINT(x fx) + 2^(nb-1), fx = (2^(nb-1)-1)/scale, packed
  high part first; the reader decodes (nx-1) icompr values.
* wr30wfn_utils.mod.F90:569-693 ...... section 10 ('NIL'): irecord = 2n+1,
  (n, ngwks, icompr, scale = max |component|), then the per-state records.
* wv30_utils.mod.F90:856-895 ......... section 23: nkpts records of the
  occupations; section 24: amu, then nkpts records of eigenvalues.
* wfnio_utils.mod.F90:130-135 ........ scale = |c| of the element with the
  largest |Re| + |Im| (izamax).
* rv30_utils.mod.F90:290-640 ......... the reader: sections taken in order,
  unwanted ones skipped record by record (utils.mod.F90:462-485, fskip) or, in
  a STREAM file, by seeking to fpos.
"""
from __future__ import annotations

import struct

import numpy as np

HEADER = " STUTTGART VERSION 3.0"


# ------------------------------------------------------------------ writing
class _W:
    def __init__(self, stream: bool):
        self.stream = stream
        self.parts: list[bytes] = []

    def rec(self, data: bytes):
        if self.stream:
            self.parts.append(data)
        else:
            n = struct.pack("<i", len(data))
            self.parts.append(n + data + n)

    def section(self, irecord: int, body=()):
        # STREAM: fpos = 1-based position right after the section
        if not self.stream:
            self.rec(struct.pack("<iq", irecord, 0))
            for b in body:
                self.rec(b)
            return
        size = 12 + sum(len(b) for b in body)
        start = sum(len(p) for p in self.parts)
        self.rec(struct.pack("<iq", irecord, start + size + 1))
        for b in body:
            self.rec(b)

    def bytes(self) -> bytes:
        return b"".join(self.parts)


def izamax_scale(c: np.ndarray) -> float:
    flat = np.asfortranarray(c).reshape(-1, order="F")
    k = int(np.argmax(np.abs(flat.real) + np.abs(flat.imag)))
    return float(abs(flat[k]))


def pack_state(a: np.ndarray, icompr: int, scale: float) -> tuple[int, np.ndarray]:
    """compress.F90 of one state's real view (2 ngw doubles): (nx, 32-bit words)."""
    n = a.size
    if icompr == 1:
        return n, np.frombuffer(a.astype("<f8").tobytes(), dtype="<u4").copy()
    nb = 64 // icompr
    k = 32 // nb  # values per word
    m = n + n % (2 * k) if k > 1 else n + n % 2
    fx = (2.0 ** (nb - 1) - 1.0) / scale
    vals = np.zeros(m, dtype=np.int64)
    vals[:n] = np.sign(a * fx) * np.floor(np.abs(a * fx) + 0.5)  # NINT
    u = (vals + 2 ** (nb - 1)) % (1 << nb) if nb < 32 else (vals + 2 ** 31) % (1 << 32)
    u = u.astype(np.uint64)
    words = np.zeros(m // k, dtype=np.uint64)
    for j in range(k):
        words |= u[j::k] << np.uint64(nb * (k - 1 - j))
    nx = m // (2 * k) if k > 1 else m // 2
    return nx, words[: 2 * nx].astype("<u4")


def write(path, c0, *, na, tau0, ecut, nel, nr, celldm, taum=None, taui=None, ibrav=1, indpg=0, cdual=4.0,
          dual=False, ngwls=0, nhgs=0, nhgls=0, icompr=1, stream=False, f=None, eigv=None, amu=0.0,
          fill=None, cm=None):
    """fill: {section: [record bytes, ...]} for sections 10-22 (a reader must skip them)."""
    c = np.asfortranarray(np.asarray(c0, dtype=np.complex128))
    ngw, nstate = c.shape
    na = np.asarray(na, dtype=np.int32)
    tau0 = np.asarray(tau0, dtype=np.float64).reshape(-1, 3)
    w = _W(stream)
    w.rec((HEADER + (" STREAM" if stream else "")).ljust(80).encode())
    w.section(2, [struct.pack("<ii", ibrav, indpg), np.asarray(celldm, "<f8").tobytes()])
    w.section(2, [struct.pack("<i", len(na)), na.astype("<i4").tobytes()])
    for t in (tau0, taum, taui):
        if t is None:
            w.section(0)
        else:
            t = np.asarray(t, dtype=np.float64).reshape(-1, 3)
            w.section(t.shape[0], [t[i].astype("<f8").tobytes() for i in range(t.shape[0])])
    nr1, nr2, nr3 = (nr, nr, nr) if np.isscalar(nr) else nr
    w.section(1, [struct.pack("<ddiiiii", ecut, cdual, 1 if dual else 0, nel, nr1, nr2, nr3)])
    w.section(1, [struct.pack("<iiiiii", nstate, 0, ngw, ngwls, nhgs, nhgls)])
    scale = izamax_scale(c)
    body = [struct.pack("<i", 1), struct.pack("<iiid", nstate, ngw, icompr, scale), struct.pack("<iii", 0, 0, 0)]
    for s in range(nstate):
        real = np.empty(2 * ngw)
        real[0::2], real[1::2] = c[:, s].real, c[:, s].imag
        nx, words = pack_state(real, icompr, scale)
        body += [struct.pack("<i", nx), words.tobytes()]
    if stream:
        w.section(-(2 * nstate + 3), body)
    else:
        w.rec(struct.pack("<iq", -(2 * nstate + 3), -1))
        for b in body:
            w.rec(b)
    if cm is not None:
        cmf = np.asfortranarray(np.asarray(cm, dtype=np.complex128))
        sc = float(np.abs(np.concatenate([cmf.real.ravel(), cmf.imag.ravel()])).max())
        body = [struct.pack("<iiid", nstate, ngw, icompr, sc)]
        for s_ in range(nstate):
            real = np.empty(2 * ngw)
            real[0::2], real[1::2] = cmf[:, s_].real, cmf[:, s_].imag
            nx, words = pack_state(real, icompr, sc)
            body += [struct.pack("<i", nx), words.tobytes()]
        w.section(2 * nstate + 1, body)
    else:
        body = (fill or {}).get(10, [])
        w.section(len(body), body)
    for sec in range(11, 23):
        body = (fill or {}).get(sec, [])
        w.section(len(body), body)
    w.section(1, [np.asarray(f, "<f8").tobytes()]) if f is not None else w.section(0)
    if eigv is not None:
        w.section(2, [struct.pack("<d", amu), np.asarray(eigv, "<f8").tobytes()])
    else:
        w.section(0)
    for _ in range(25, 100):
        w.section(0)
    with open(path, "wb") as f:
        f.write(w.bytes())
    return scale


# ------------------------------------------------------------------ reading
class _R:
    def __init__(self, data: bytes):
        self.d = data
        self.p = 0
        self.stream = struct.unpack_from("<i", data, 0)[0] != 80

    def rec(self, want: int | None = None) -> bytes:
        if self.stream:
            b = self.d[self.p:self.p + want]
            if len(b) != want:
                raise EOFError("short STREAM read")
            self.p += want
            return b
        (n,) = struct.unpack_from("<i", self.d, self.p)
        b = self.d[self.p + 4:self.p + 4 + n]
        (t,) = struct.unpack_from("<i", self.d, self.p + 4 + n)
        if n < 0 or t != n or len(b) != n:
            raise ValueError("bad record frame")
        self.p += 8 + n
        return b

    def section(self):
        b = self.rec(12)
        irecord = struct.unpack_from("<i", b, 0)[0]
        fpos = struct.unpack_from("<q", b, 4)[0] if len(b) >= 12 else 0
        return irecord, fpos

    def skip(self, irecord, fpos):
        if self.stream:
            self.p = fpos - 1
        else:
            for _ in range(abs(irecord)):
                self.rec()


def unpack_state(words: np.ndarray, nx: int, icompr: int, scale: float) -> np.ndarray:
    """decompr + sunpack of compress.F90 (the Linux variant)."""
    if icompr == 1:
        return np.frombuffer(words.astype("<u4").tobytes(), dtype="<f8")[:nx].copy()
    nb = 64 // icompr
    k = 32 // nb
    n = (nx - 1) * icompr
    fx = scale / (2.0 ** (nb - 1) - 1.0)
    w = words.astype(np.uint64)
    vals = np.empty(len(w) * k, dtype=np.int64)
    for j in range(k):
        vals[j::k] = ((w >> np.uint64(nb * (k - 1 - j))) & np.uint64((1 << nb) - 1)).astype(np.int64)
    vals = vals[:n] - 2 ** (nb - 1)
    return vals.astype(np.float64) * fx


def read(path) -> dict:
    with open(path, "rb") as f:
        r = _R(f.read())
    out = {"stream": r.stream}
    hdr = r.rec(80).decode(errors="replace")
    if "STUTTGART" not in hdr:
        raise ValueError("not a RESTART file")
    irec, fpos = r.section()
    if irec == 2:
        out["ibrav"], out["indpg"] = struct.unpack("<ii", r.rec(8)[:8])
        out["celldm"] = np.frombuffer(r.rec(48)[:48], "<f8").copy()
    else:
        r.skip(irec, fpos)
    irec, fpos = r.section()
    if irec == 2:
        (nsp,) = struct.unpack("<i", r.rec(4)[:4])
        out["na"] = np.frombuffer(r.rec(4 * nsp)[:4 * nsp], "<i4").copy()
    else:
        r.skip(irec, fpos)
    nat = int(out["na"].sum()) if "na" in out else 0
    for key in ("tau0", "taum", "taui"):
        irec, fpos = r.section()
        if irec == nat and irec > 0:
            out[key] = np.array([np.frombuffer(r.rec(24)[:24], "<f8") for _ in range(nat)])
        else:
            r.skip(irec, fpos)
    irec, fpos = r.section()
    if irec == 1:
        ecut, cdual, dual, nel, n1, n2, n3 = struct.unpack("<ddiiiii", r.rec(36)[:36])
        out.update(ecut=ecut, cdual=cdual, dual=bool(dual), nel=nel, nr=(n1, n2, n3))
    else:
        r.skip(irec, fpos)
    irec, fpos = r.section()
    if irec == 1:
        n, nk, ngwks, ngwls, nhgs, nhgls = struct.unpack("<iiiiii", r.rec(24)[:24])
        out.update(nstate=n, nkpts=nk, ngwks=ngwks, ngwls=ngwls, nhgs=nhgs, nhgls=nhgls)
    else:
        r.skip(irec, fpos)
    irec, fpos = r.section()
    if irec < 0:
        (iwfntype,) = struct.unpack("<i", r.rec(4)[:4])
        n0, ngwks0, icompr, scale = struct.unpack("<iiid", r.rec(20)[:20])
        r.rec(12)
        c = np.zeros((ngwks0, n0), dtype=np.complex128, order="F")
        for s in range(n0):
            (nx,) = struct.unpack("<i", r.rec(4)[:4])
            words = np.frombuffer(r.rec(8 * nx)[:8 * nx], "<u4")
            a = np.zeros(2 * ngwks0)
            v = unpack_state(words, nx, icompr, scale)
            a[:len(v)] = v
            c[:, s] = a[0::2] + 1j * a[1::2]
        out.update(iwfntype=iwfntype, icompr=icompr, scale=scale, c0=c)
    if r.p >= len(r.d):
        return out
    irec, fpos = r.section()
    if irec > 0:
        n0, ngwks0, icompr, scale = struct.unpack("<iiid", r.rec(20)[:20])
        cmv = np.zeros((ngwks0, n0), dtype=np.complex128, order="F")
        for s in range(n0):
            (nx,) = struct.unpack("<i", r.rec(4)[:4])
            words = np.frombuffer(r.rec(8 * nx)[:8 * nx], "<u4")
            a = np.zeros(2 * ngwks0)
            v = unpack_state(words, nx, icompr, scale)
            a[:len(v)] = v
            cmv[:, s] = a[0::2] + 1j * a[1::2]
        out.update(cm=cmv, cm_scale=scale)
    else:
        r.skip(irec, fpos)
    for _ in range(11, 23):
        irec, fpos = r.section()
        r.skip(irec, fpos)
    n = out.get("nstate", 0)
    irec, fpos = r.section()
    if irec >= 1:
        out["f"] = np.frombuffer(r.rec(8 * n)[:8 * n], "<f8").copy()
        r.skip(irec - 1, fpos) if not r.stream else None
    irec, fpos = r.section()
    if irec >= 2:
        (out["amu"],) = struct.unpack("<d", r.rec(8)[:8])
        out["eigv"] = np.frombuffer(r.rec(8 * n)[:8 * n], "<f8").copy()
    return out
