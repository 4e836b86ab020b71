"""A small JPEG encoder (ITU-T T.81) for the decoder's tests: baseline and
progressive Huffman processes, Huffman tables built from the symbol counts
of each scan (Annex K.2, code lengths limited to 16 bits), any sampling
factors, restart intervals. Test infrastructure only.

`encode` returns the file bytes and the quantised coefficients it coded;
`reconstruct` turns those coefficients into the image a decoder following
T.81 A.3.3 exactly (double-precision IDCT, centred linear upsampling, JFIF
colour equations) produces.
"""
import heapq

import numpy as np


def zigzag():
    """Zig-zag position -> row-major index of the 8x8 block."""
    order = []
    for s in range(15):
        rows = range(max(0, s - 7), min(s, 7) + 1)
        rows = reversed(list(rows)) if s % 2 == 0 else rows
        order += [r * 8 + (s - r) for r in rows]
    return order


ZZ = zigzag()
# C[x, u] = C(u)/2 cos((2x + 1) u pi / 16); orthonormal, so F = C^T f C and f = C F C^T
_C = np.array([[(np.sqrt(0.5) if u == 0 else 1.0) * 0.5 * np.cos((2 * x + 1) * u * np.pi / 16) for u in range(8)]
               for x in range(8)])


def quant_table(scale):
    """A smooth quantisation table (row-major), larger steps at high frequency."""
    v, u = np.mgrid[0:8, 0:8]
    return np.clip(np.round(1 + scale * (u + v)), 1, 255).astype(np.int64)


def _to_planes(img, ycc):
    img = np.asarray(img)
    if img.ndim == 2:
        return [img.astype(np.float64)]
    r, g, b = [img[..., k].astype(np.float64) for k in range(3)]
    if not ycc:
        return [r, g, b]
    y = 0.299 * r + 0.587 * g + 0.114 * b
    cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128.0
    cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128.0
    return [np.clip(np.round(p), 0, 255) for p in (y, cb, cr)]


def _component_dims(w, h, hs, vs, hmax, vmax):
    cw = -(-w * hs // hmax)
    ch = -(-h * vs // vmax)
    return cw, ch


def _coefficients(planes, w, h, sampling, qts):
    hmax = max(s[0] for s in sampling)
    vmax = max(s[1] for s in sampling)
    mcux = -(-w // (8 * hmax))
    mcuy = -(-h // (8 * vmax))
    out = []
    for p, (hs, vs), q in zip(planes, sampling, qts):
        fx, fy = hmax // hs, vmax // vs
        cw, ch = _component_dims(w, h, hs, vs, hmax, vmax)
        # box-filter down to the component's size (edge pixels replicated)
        ph = np.pad(p, ((0, ch * fy - h), (0, cw * fx - w)), mode="edge")
        sub = ph.reshape(ch, fy, cw, fx).mean(axis=(1, 3))
        bw, bh = mcux * hs, mcuy * vs
        full = np.pad(sub, ((0, bh * 8 - ch), (0, bw * 8 - cw)), mode="edge") - 128.0
        blocks = full.reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3)
        F = np.einsum("xu,abxy,yv->abuv", _C, blocks, _C)  # F[.., u(row), v(col)] in row-major order
        coef = np.round(F / q).astype(np.int64).reshape(bh, bw, 64)
        out.append(dict(coef=coef, hs=hs, vs=vs, cw=cw, ch=ch, bw=bw, bh=bh, cbw=-(-cw // 8), cbh=-(-ch // 8), q=q))
    return out, hmax, vmax, mcux, mcuy


def reconstruct(comps, w, h, hmax, vmax, ycc):
    """The image an exact T.81 decoder produces from these coefficients."""
    planes = []
    for c in comps:
        F = (c["coef"] * c["q"].reshape(64)).reshape(c["bh"], c["bw"], 8, 8).astype(np.float64)
        f = np.einsum("yv,abvu,xu->abyx", _C, F, _C)
        pl = np.clip(np.floor(f + 128.0 + 0.5), 0, 255).transpose(0, 2, 1, 3).reshape(c["bh"] * 8, c["bw"] * 8)
        fx, fy = hmax // c["hs"], vmax // c["vs"]
        planes.append(_upsample(pl, c["cw"], c["ch"], fx, fy, w, h))
    if len(planes) == 1:
        return np.repeat(planes[0][..., None], 3, axis=2).astype(np.uint8)
    if not ycc:
        return np.stack(planes, -1).astype(np.uint8)
    y, cb, cr = planes[0], planes[1] - 128.0, planes[2] - 128.0
    rgb = [y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb]
    return np.stack([np.clip(np.floor(v + 0.5), 0, 255) for v in rgb], -1).astype(np.uint8)


def _upsample(pl, cw, ch, fx, fy, w, h):
    def axis(n_out, f, n):
        i = np.arange(n_out)
        if f == 1:
            return i, i, np.zeros(n_out)
        s = (i + 0.5) / f - 0.5
        fl = np.floor(s)
        i0 = np.clip(fl.astype(int), 0, n - 1)
        i1 = np.clip(fl.astype(int) + 1, 0, n - 1)
        return i0, i1, s - fl
    if fx == 1 and fy == 1:
        return pl[:h, :w]
    x0, x1, wx = axis(w, fx, cw)
    y0, y1, wy = axis(h, fy, ch)
    top = pl[y0][:, x0] * (1 - wx) + pl[y0][:, x1] * wx
    bot = pl[y1][:, x0] * (1 - wx) + pl[y1][:, x1] * wx
    v = top * (1 - wy)[:, None] + bot * wy[:, None]
    return np.clip(np.floor(v + 0.5), 0, 255)


# ---------------------------------------------------------------- entropy coding
class _Writer:
    def __init__(self):
        self.out = bytearray()
        self.acc = 0
        self.n = 0

    def bits(self, value, n):
        if n == 0:
            return
        self.acc = (self.acc << n) | (value & ((1 << n) - 1))
        self.n += n
        while self.n >= 8:
            b = (self.acc >> (self.n - 8)) & 0xFF
            self.out.append(b)
            if b == 0xFF:
                self.out.append(0)
            self.n -= 8
            self.acc &= (1 << self.n) - 1

    def align(self):
        if self.n:
            self.bits((1 << (8 - self.n)) - 1, 8 - self.n)


def build_table(freq):
    """Symbol counts -> (BITS[1..16], HUFFVAL) per T.81 K.2, with the
    all-ones code point reserved."""
    syms = sorted(s for s, c in freq.items() if c > 0) or [0]
    items = [(freq.get(s, 1), s) for s in syms] + [(1, 256)]
    heap = [(c, i, [s]) for i, (c, s) in enumerate(items)]
    heapq.heapify(heap)
    size = {s: 0 for _, s in items}
    k = len(heap)
    while len(heap) > 1:
        c1, _, a = heapq.heappop(heap)
        c2, _, b = heapq.heappop(heap)
        for s in a + b:
            size[s] += 1
        heapq.heappush(heap, (c1 + c2, k, a + b))
        k += 1
    bits = [0] * 40
    for s in size:
        bits[size[s]] += 1
    i = 39
    while i > 16:
        while bits[i] > 0:
            j = i - 2
            while bits[j] == 0:
                j -= 1
            bits[i] -= 2
            bits[i - 1] += 1
            bits[j + 1] += 2
            bits[j] -= 1
        i -= 1
    while bits[i] == 0:
        i -= 1
    bits[i] -= 1  # the reserved code point
    vals = [s for _, s in sorted((size[s], s) for s in syms)]
    return bits[1:17], vals


def _codes(bits, vals):
    codes, code, k = {}, 0, 0
    for l in range(1, 17):
        for _ in range(bits[l - 1]):
            codes[vals[k]] = (code, l)
            code += 1
            k += 1
        code <<= 1
    return codes


def _cat(v):
    return int(abs(v)).bit_length()


def _vbits(v, s):
    return v if v >= 0 else v + (1 << s) - 1


class _Scan:
    """Records a scan as operations, so the same pass serves for the
    symbol counts and for the coded bits."""

    def __init__(self):
        self.ops = []

    def sym(self, cls, tid, s):
        self.ops.append((0, cls, tid, s))

    def bits(self, v, n):
        if n:
            self.ops.append((1, v, n))

    def restart(self):
        self.ops.append((2,))


def _seq_block(S, b, pred, tdc, tac):
    diff = int(b[0]) - pred
    s = _cat(diff)
    S.sym(0, tdc, s)
    S.bits(_vbits(diff, s), s)
    r = 0
    zz = [int(b[ZZ[k]]) for k in range(64)]
    last = max([k for k in range(1, 64) if zz[k] != 0], default=0)
    for k in range(1, last + 1):
        v = zz[k]
        if v == 0:
            r += 1
            continue
        while r > 15:
            S.sym(1, tac, 0xF0)
            r -= 16
        s = _cat(v)
        S.sym(1, tac, (r << 4) | s)
        S.bits(_vbits(v, s), s)
        r = 0
    if last < 63:
        S.sym(1, tac, 0x00)
    return int(b[0])


class _EobState:
    def __init__(self):
        self.run = 0
        self.be = []

    def flush(self, S, tac):
        if self.run:
            nb = self.run.bit_length() - 1
            S.sym(1, tac, nb << 4)
            S.bits(self.run - (1 << nb), nb)
            for bit in self.be:
                S.bits(bit, 1)
        self.run = 0
        self.be = []


def _ac_first(S, b, ss, se, al, tac, eob):
    vals = []
    for k in range(ss, se + 1):
        c = int(b[ZZ[k]])
        m = abs(c) >> al
        vals.append(m if c >= 0 else -m)
    nz = [i for i, v in enumerate(vals) if v]
    if not nz:
        eob.run += 1
        if eob.run == 0x7FFF:
            eob.flush(S, tac)
        return
    eob.flush(S, tac)
    r = 0
    for i in range(nz[-1] + 1):
        v = vals[i]
        if v == 0:
            r += 1
            continue
        while r > 15:
            S.sym(1, tac, 0xF0)
            r -= 16
        s = _cat(v)
        S.sym(1, tac, (r << 4) | s)
        S.bits(_vbits(v, s), s)
        r = 0
    if nz[-1] < len(vals) - 1:
        eob.run += 1
        if eob.run == 0x7FFF:
            eob.flush(S, tac)


def _ac_refine(S, b, ss, se, al, tac, eob):
    absv = [abs(int(b[ZZ[k]])) >> al for k in range(ss, se + 1)]
    sign = [int(b[ZZ[k]]) > 0 for k in range(ss, se + 1)]
    last_new = max([i for i, t in enumerate(absv) if t == 1], default=-1)
    r, br = 0, []
    for i, t in enumerate(absv):
        if t == 0:
            r += 1
            continue
        while r > 15 and i <= last_new:
            eob.flush(S, tac)
            S.sym(1, tac, 0xF0)
            for bit in br:
                S.bits(bit, 1)
            br = []
            r -= 16
        if t > 1:
            br.append(t & 1)
            continue
        eob.flush(S, tac)
        S.sym(1, tac, (r << 4) | 1)
        S.bits(1 if sign[i] else 0, 1)
        for bit in br:
            S.bits(bit, 1)
        br, r = [], 0
    if r > 0 or br:
        eob.run += 1
        eob.be += br
        if eob.run == 0x7FFF:
            eob.flush(S, tac)


def _marker(out, m, payload=b""):
    out += bytes([0xFF, m])
    if m not in (0xD8, 0xD9):
        out += (len(payload) + 2).to_bytes(2, "big") + payload


def encode(img, sampling=None, qscale=1.0, progressive=False, restart=0, interleave=True, ycc=True,
           script=None, ids=None, adobe=None):
    """img: (h, w) or (h, w, 3) uint8. Returns (bytes, comps, hmax, vmax)."""
    img = np.asarray(img)
    h, w = img.shape[:2]
    planes = _to_planes(img, ycc)
    nc = len(planes)
    sampling = sampling or [(1, 1)] * nc
    qts = [quant_table(qscale), quant_table(qscale * 1.5)]
    tq = [0] + [1] * (nc - 1)
    comps, hmax, vmax, mcux, mcuy = _coefficients(planes, w, h, sampling, [qts[t] for t in tq])
    ids = ids or list(range(1, nc + 1))
    out = bytearray()
    _marker(out, 0xD8)
    if adobe is not None:
        _marker(out, 0xEE, b"Adobe" + bytes([0, 100, 0, 0, 0, 0, adobe]))
    for t in range(2 if nc > 1 else 1):
        q = qts[t].reshape(64)
        _marker(out, 0xDB, bytes([t]) + bytes(int(q[ZZ[k]]) for k in range(64)))
    sof = bytes([8]) + h.to_bytes(2, "big") + w.to_bytes(2, "big") + bytes([nc])
    for i in range(nc):
        sof += bytes([ids[i], (sampling[i][0] << 4) | sampling[i][1], tq[i]])
    _marker(out, 0xC2 if progressive else 0xC0, sof)
    if restart:
        _marker(out, 0xDD, restart.to_bytes(2, "big"))
    tid = [0] + [1] * (nc - 1)
    if progressive:
        script = script or default_script(nc)
    else:
        script = [(list(range(nc)), 0, 63, 0, 0)] if interleave else [([c], 0, 63, 0, 0) for c in range(nc)]
    for comp_ids, ss, se, ah, al in script:
        S = _Scan()
        preds = {c: 0 for c in comp_ids}
        eob = _EobState()

        def unit(ci, bx, by):
            c = comps[ci]
            b = c["coef"][by, bx]
            if not progressive:
                preds[ci] = _seq_block(S, b, preds[ci], tid[ci], tid[ci])
            elif ss == 0 and ah == 0:
                v = int(b[0]) >> al
                diff = v - preds[ci]
                preds[ci] = v
                s = _cat(diff)
                S.sym(0, tid[ci], s)
                S.bits(_vbits(diff, s), s)
            elif ss == 0:
                S.bits((int(b[0]) >> al) & 1, 1)
            elif ah == 0:
                _ac_first(S, b, ss, se, al, tid[ci], eob)
            else:
                _ac_refine(S, b, ss, se, al, tid[ci], eob)

        if len(comp_ids) == 1:
            c = comps[comp_ids[0]]
            units = [[(comp_ids[0], i % c["cbw"], i // c["cbw"])] for i in range(c["cbw"] * c["cbh"])]
        else:
            units = []
            for m in range(mcux * mcuy):
                mx, my = m % mcux, m // mcux
                u = []
                for ci in comp_ids:
                    c = comps[ci]
                    u += [(ci, mx * c["hs"] + x, my * c["vs"] + y) for y in range(c["vs"]) for x in range(c["hs"])]
                units.append(u)
        for k, u in enumerate(units):
            for args in u:
                unit(*args)
            if restart and (k + 1) % restart == 0 and k + 1 < len(units):
                if progressive and ss > 0:
                    eob.flush(S, tid[comp_ids[0]])
                S.restart()
                for ci in comp_ids:
                    preds[ci] = 0
        if progressive and ss > 0:
            eob.flush(S, tid[comp_ids[0]])
        # tables from this scan's counts, then the coded scan
        freq = {}
        for op in S.ops:
            if op[0] == 0:
                freq.setdefault((op[1], op[2]), {}).setdefault(op[3], 0)
                freq[(op[1], op[2])][op[3]] += 1
        codes = {}
        for (cls, t), f in sorted(freq.items()):
            bits, vals = build_table(f)
            codes[(cls, t)] = _codes(bits, vals)
            _marker(out, 0xC4, bytes([(cls << 4) | t]) + bytes(bits) + bytes(vals))
        sos = bytes([len(comp_ids)])
        for ci in comp_ids:
            sos += bytes([ids[ci], (tid[ci] << 4) | tid[ci]])
        sos += bytes([ss, se, (ah << 4) | al])
        _marker(out, 0xDA, sos)
        W = _Writer()
        rst = 0
        for op in S.ops:
            if op[0] == 0:
                code, l = codes[(op[1], op[2])][op[3]]
                W.bits(code, l)
            elif op[0] == 1:
                W.bits(op[1], op[2])
            else:
                W.align()
                W.out += bytes([0xFF, 0xD0 + rst])
                rst = (rst + 1) & 7
        W.align()
        out += W.out
    _marker(out, 0xD9)
    return bytes(out), comps, hmax, vmax


def default_script(nc):
    """A progression with every kind of scan: DC first and refinement, AC
    spectral bands, AC successive-approximation refinements."""
    s = [(list(range(nc)), 0, 0, 0, 1)]
    for c in range(nc):
        s.append(([c], 1, 5, 0, 2))
    for c in range(nc):
        s.append(([c], 6, 63, 0, 2))
    s.append((list(range(nc)), 0, 0, 1, 0))
    for c in range(nc):
        s.append(([c], 1, 63, 2, 1))
    for c in range(nc):
        s.append(([c], 1, 63, 1, 0))
    return s
