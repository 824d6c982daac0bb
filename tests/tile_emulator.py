"""Test infrastructure: a numpy restatement of how the tile kernels interpret
an encoded tile plan (aqsg_debug_tile_plan), used to check the host encoder
(pass planning, register phases, control masks, matrix layouts, tensor-core
operands and index tables) on the CPU against the FP64 oracle.  It restates the record semantics of
afquantumsim_gb300/csrc/tile_device.cuh (tile_run_ops, rphase_run) — the
device code itself runs only in the GPU tests."""
import numpy as np

# tile op classes and register-op kinds / flags (tile_device.cuh, aqsg_internal.h)
L_PERM_X, L_PERM_OR, L_PERM_SWAP, L_DIAG1, L_DIAG2, L_MAT2, L_MATK, T_RPHASE = 1, 2, 3, 4, 5, 6, 7, 8
RK_MAT2C, RK_MAT2R, RK_PERM, RK_SWAP, RK_DIAG, RK_DIAGR, RK_MATK = 1, 2, 3, 4, 5, 6, 7
RF_EXT, RF_OR, RF_TTHR, RF_TEXT = 1 << 16, 1 << 17, 1 << 18, 1 << 19

TILE_OP = np.dtype([("cls", "<i4"), ("lt0", "<i4"), ("lt1", "<i4"), ("k", "<i4"), ("ltb", "<i4", 5),
                    ("mat", "<i4"), ("ext_t", "<i4"), ("pad", "<i4"), ("cm_loc", "<u8"), ("cv_loc", "<u8"),
                    ("cm_ext", "<u8"), ("cv_ext", "<u8"), ("am_loc", "<u8"), ("am_ext", "<u8"), ("m", "<f8", 8)])
R_OP = np.dtype([("code", "<u4"), ("ctl", "<u4"), ("em", "<u4"), ("extra", "<u4"), ("cm_ext", "<u8"),
                 ("cv_ext", "<u8"), ("am_ext", "<u8"), ("ext_t", "<i4"), ("amt", "<u4"), ("coef", "u1", 112)])
assert TILE_OP.itemsize == 160 and R_OP.itemsize == 160


def _coefs(raw: bytes, count: int, c64: bool) -> np.ndarray:
    """count complex values stored in the kernel's type"""
    if c64:
        f = np.frombuffer(raw, dtype="<f4", count=2 * count).astype(np.float64)
    else:
        f = np.frombuffer(raw, dtype="<f8", count=2 * count)
    return f[0::2] + 1j * f[1::2]


def _reals(raw: bytes, count: int, c64: bool) -> np.ndarray:
    return np.frombuffer(raw, dtype="<f4" if c64 else "<f8", count=count).astype(np.float64)


def _tile_coef(m: np.ndarray, i: int, c64: bool) -> complex:
    """ld_coef<T>: the double coefficient as the kernel's type"""
    re, im = m[2 * i], m[2 * i + 1]
    if c64:
        re, im = float(np.float32(re)), float(np.float32(im))
    return complex(re, im)


def _pool_matrix(pool: bytes, off: int, d: int, c64: bool) -> np.ndarray:
    return _coefs(pool[off:off + (8 if c64 else 16) * d * d], d * d, c64).reshape(d, d)


def _pairs(X, j0, j1, cond, m00, m01, m10, m11):
    a, b = X[:, j0].copy(), X[:, j1].copy()
    X[:, j0] = np.where(cond, m00 * a + m01 * b, a)
    X[:, j1] = np.where(cond, m10 * a + m11 * b, b)


def _swap(X, j0, j1, cond):
    a, b = X[:, j0].copy(), X[:, j1].copy()
    X[:, j0] = np.where(cond, b, a)
    X[:, j1] = np.where(cond, a, b)


def _tile_op(X, base, j, op, pool, c64):
    cls = int(op["cls"])
    cm, cv = int(op["cm_loc"]), int(op["cv_loc"])
    ext = ((base & np.uint64(op["cm_ext"])) == np.uint64(op["cv_ext"]))[:, None]
    if cls in (L_DIAG1, L_DIAG2):
        ph0, ph1 = _tile_coef(op["m"], 0, c64), _tile_coef(op["m"], 1, c64)
        sel = (j & cm) == cv
        if cls == L_DIAG2 and op["lt0"] >= 0:
            ph = np.where((j >> int(op["lt0"])) & 1, ph1, ph0)[None, :]
        elif cls == L_DIAG2:
            ph = np.where((base >> np.uint64(op["ext_t"])) & np.uint64(1), ph1, ph0)[:, None]
        else:
            ph = ph0
        X[:] = np.where(ext & sel[None, :], X * ph, X)
        return
    if cls in (L_MAT2, L_PERM_X, L_PERM_OR):
        t = 1 << int(op["lt0"])
        j0 = j[(j & t) == 0]
        cond = ext & ((j0 & cm) == cv)[None, :]
        if cls == L_MAT2:
            c = [_tile_coef(op["m"], i, c64) for i in range(4)]
            _pairs(X, j0, j0 | t, cond, *c)
        else:
            if cls == L_PERM_OR:
                or_all = ((base & np.uint64(op["am_ext"])) != 0)[:, None]
                cond = cond & (or_all | ((j0 & int(op["am_loc"])) != 0)[None, :])
            _swap(X, j0, j0 | t, cond)
        return
    if cls == L_PERM_SWAP:
        ma, mb = 1 << int(op["lt0"]), 1 << int(op["lt1"])
        js = j[((j & ma) == 0) & ((j & mb) != 0)]
        cond = ext & ((js & cm) == cv)[None, :]
        _swap(X, js, js ^ (ma | mb), cond)
        return
    if cls == L_MATK:
        k = int(op["k"])
        d = 1 << k
        ltb = [int(b) for b in op["ltb"][:k]]
        tm = sum(1 << b for b in ltb)
        off = np.array([sum(((r >> (k - 1 - i)) & 1) << ltb[i] for i in range(k)) for r in range(d)])
        jb = j[(j & tm) == 0]
        cond = ext & ((jb & cm) == cv)[None, :]
        M = _pool_matrix(pool, int(op["mat"]), d, c64)
        V = np.stack([X[:, jb | off[c]] for c in range(d)], axis=-1)  # (T, groups, d)
        W = V @ M.T
        for r in range(d):
            X[:, jb | off[r]] = np.where(cond, W[..., r], X[:, jb | off[r]])
        return
    raise AssertionError(f"unexpected tile op class {cls}")


# tensor-core ops (tile_device.cuh tc_apply_tm, tile_kernels.cu tc_operand /
# tc_tables): in the pass's operand blob, at the op's offset, the B operand's
# BF16 hi split, its lo split (each 2N x 2K bytes, no-swizzle K-major), then
# the index tables (colbase: 512 x u16 byte offsets of the data columns in
# the padded tile, offr at +1024: the matrix rows' byte offsets)
TC_TABLE_BYTES = 1024 + 64
TC_ROW_AMPS = 34  # padded tile row: 32 amplitudes + 2 of padding (272 bytes)


def _bf16(x):
    """float32 values rounded to bfloat16 (nearest even), as float64"""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _kmajor(raw: np.ndarray, rows: int, K: int) -> np.ndarray:
    """rows x K bf16 matrix from its no-swizzle K-major byte image"""
    r, kk = np.meshgrid(np.arange(rows), np.arange(K), indexing="ij")
    off = ((r >> 3) * (K >> 3) + (kk >> 3)) * 128 + (r & 7) * 16 + (kk & 7) * 2
    h = raw[off].astype(np.uint32) | (raw[off + 1].astype(np.uint32) << 8)
    return (h << 16).astype(np.uint32).view(np.float32).astype(np.float64)


def _tc_op(X, base, op, pool, blob_at):
    """Y = U X of a fused unitary as the tensor cores compute it: the data
    split into BF16 hi + lo, products Ahi Bhi + Ahi Blo + Alo Bhi"""
    k = int(op["k"])
    d = 1 << k
    K = N = 2 * d
    split = 2 * N * K
    at = blob_at + int(op["mat"])
    raw = np.frombuffer(pool, dtype=np.uint8)
    b_hi = _kmajor(raw[at:at + split], N, K)
    b_lo = _kmajor(raw[at + split:at + 2 * split], N, K)
    tables = at + 2 * split
    cols = 4096 // d
    colbase = np.frombuffer(pool, dtype="<u2", count=cols, offset=tables).astype(np.int64)
    offr = np.frombuffer(pool, dtype="<u2", count=d, offset=tables + 1024).astype(np.int64)
    e = (colbase[:, None] + offr[None, :]) // 8  # amplitude slots in the padded tile
    J = (e // TC_ROW_AMPS) * 32 + e % TC_ROW_AMPS  # tile-local indices, (cols, d)
    x = X[:, J]
    a = np.empty(x.shape[:-1] + (K,))
    a[..., 0::2], a[..., 1::2] = x.real, x.imag
    a32 = a.astype(np.float32)
    a_hi = _bf16(a32)
    a_lo = _bf16(a32 - a_hi.astype(np.float32))
    y = a_hi @ b_hi.T + a_hi @ b_lo.T + a_lo @ b_hi.T
    ext = ((base & np.uint64(op["cm_ext"])) == np.uint64(op["cv_ext"]))[:, None, None]
    X[:, J] = np.where(ext, y[..., 0::2] + 1j * y[..., 1::2], x)


def _phase(X, base, j, head, rops, pool, c64):
    rb = int(head["lt0"])
    rpos = [(int(head["am_loc"]) >> (4 * i)) & 15 for i in range(rb)]
    rmask = sum(1 << p for p in rpos)
    all_e = (1 << (1 << rb)) - 1

    def elem(jj):  # register element index of local indices jj
        e = np.zeros_like(jj)
        for i, p in enumerate(rpos):
            e |= ((jj >> p) & 1) << i
        return e

    for r in rops:
        code = int(r["code"])
        kind, a = code & 0xFF, (code >> 8) & 0xFF
        ctl = int(r["ctl"])
        em = int(r["em"]) & all_e
        ext = np.ones((X.shape[0], 1), dtype=bool)
        if code & RF_EXT:
            ext = ((base & np.uint64(r["cm_ext"])) == np.uint64(r["cv_ext"]))[:, None]
        coef = bytes(r["coef"])

        def tcond(jj):  # control on slot-index bits
            return ((jj & ~rmask) & (ctl & 0xFFFF)) == (ctl >> 16)

        def ebit(mask, jj):
            return ((mask >> elem(jj)) & 1).astype(bool)

        if kind in (RK_MAT2C, RK_MAT2R, RK_PERM):
            t = 1 << rpos[a]
            j0 = j[(j & t) == 0]
            cond = ext & (tcond(j0) & ebit(em, j0))[None, :]
            if kind == RK_PERM:
                if code & RF_OR:
                    jt = j0 & ~rmask
                    or_t = ((jt & int(r["amt"])) != 0)[None, :] | ((base & np.uint64(r["am_ext"])) != 0)[:, None]
                    om = ebit(int(r["em"]) >> 16, j0)[None, :]
                    cond = cond & (or_t | om)
                _swap(X, j0, j0 | t, cond)
            elif kind == RK_MAT2C:
                c = _coefs(coef, 4, c64)
                _pairs(X, j0, j0 | t, cond, *c)
            else:
                c = _reals(coef, 4, c64)
                _pairs(X, j0, j0 | t, cond, *c)
        elif kind == RK_SWAP:
            i_, j_ = a & 15, (code >> 12) & 15
            mi, mj = 1 << rpos[i_], 1 << rpos[j_]
            js = j[((j & mi) == 0) & ((j & mj) != 0)]
            cond = ext & (tcond(js) & ebit(em, js))[None, :]
            _swap(X, js, js ^ (mi | mj), cond)
        elif kind in (RK_DIAG, RK_DIAGR):
            c0, c1 = _coefs(coef, 2, c64)
            cond = ext & (tcond(j) & ebit(em, j))[None, :]
            if kind == RK_DIAGR:
                ph = np.where((elem(j) >> a) & 1, c1, c0)[None, :]
            elif code & RF_TTHR:
                ph = np.where((j >> int(r["extra"])) & 1, c1, c0)[None, :]
            elif code & RF_TEXT:
                ph = np.where((base >> np.uint64(r["ext_t"])) & np.uint64(1), c1, c0)[:, None]
            else:
                ph = c0
            X[:] = np.where(cond, X * ph, X)
        elif kind == RK_MATK:
            rm = a
            regs = [i for i in range(rb) if (rm >> i) & 1]
            k = len(regs)
            d = 1 << k
            off = np.array([sum(((rr >> b) & 1) << rpos[regs[b]] for b in range(k)) for rr in range(d)])
            tmask = sum(1 << rpos[i] for i in regs)
            jb = j[(j & tmask) == 0]
            cond = ext & (tcond(jb) & ebit(em, jb))[None, :]
            M = _pool_matrix(pool, int(r["extra"]), d, c64)
            V = np.stack([X[:, jb | off[c]] for c in range(d)], axis=-1)
            W = V @ M.T
            for rr in range(d):
                X[:, jb | off[rr]] = np.where(cond, W[..., rr], X[:, jb | off[rr]])
        else:
            raise AssertionError(f"unexpected register op kind {kind}")


def run_plan(psi: np.ndarray, n: int, passes, table: bytes, pool: bytes, c64: bool) -> np.ndarray:
    """Apply an encoded plan to the complex128 state psi (copy returned)."""
    psi = psi.copy()
    recs = np.frombuffer(table, dtype=TILE_OP)
    rrecs = np.frombuffer(table, dtype=R_OP)
    for p in passes:
        m = p.m
        tb = [int(p.tbits[i]) for i in range(m)]
        other = [b for b in range(n) if b not in tb]
        tiles = 1 << (n - m)
        t = np.arange(tiles, dtype=np.uint64)
        base = np.zeros(tiles, dtype=np.uint64)
        for i, b in enumerate(other):
            base |= ((t >> np.uint64(i)) & np.uint64(1)) << np.uint64(b)
        j = np.arange(1 << m, dtype=np.int64)
        loc = np.zeros(1 << m, dtype=np.uint64)
        for i, b in enumerate(tb):
            loc |= ((j.astype(np.uint64) >> np.uint64(i)) & np.uint64(1)) << np.uint64(b)
        G = (base[:, None] | loc[None, :]).astype(np.int64)
        X = psi[G]
        q = p.first
        end = p.first + p.count
        while q < end:
            op = recs[q]
            if int(op["cls"]) == T_RPHASE:
                _phase(X, base, j, op, rrecs[q + 1:q + 1 + int(op["k"])], pool, c64)
                q += 1 + int(op["k"])
            elif int(op["cls"]) == L_MATK and int(op["pad"]) and getattr(p, "tc", 0):
                _tc_op(X, base, op, pool, int(p.tc_blob))
                q += 1
            else:
                _tile_op(X, base, j, op, pool, c64)
                q += 1
        psi[G] = X
    return psi
