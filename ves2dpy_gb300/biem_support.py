"""Far field between vesicles and near-zone bookkeeping on the device
(reference: mytorch/biem_support.py)."""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _native as nat
from .layout import as_device_f64, from_vm, to_vm


def _i32(n, device):
    return torch.zeros(max(int(n), 1), dtype=torch.int32, device=device)


class NearZone:
    """Device near-pair lists (replaces the NearV2V tuple of naiveNearZoneInfo,
    biem_support.py:520-613, and the NearStruct of matlab getZone).

    ``scheme`` is ``"py_hh"`` or ``"matlab"``.  Indexing with 2, 3, 4 (or -1)
    returns the reference's index tuples ``(id1, id2)``, ``(id1_hh, id2_hh)``
    and ``(ids0, ids1, ids2)`` expanded on the host (small suspensions only).
    """

    def __init__(self, scheme, N, Nup, nv, maxc, max_entries, device):
        self.scheme, self.N, self.Nup, self.nv = scheme, N, Nup, nv
        self.maxc, self.max_entries, self.device = maxc, max_entries, device
        wN, wU = (N + 31) // 32, (Nup + 31) // 32
        self.cand_count = _i32(nv, device)
        self.cand_src = _i32(nv * maxc, device)
        self.excl_mask = _i32(nv * maxc * wN, device)
        self.hh_mask = _i32(nv * maxc * wU, device)
        self.n_entries = _i32(1, device)
        self.ent_tsj = _i32(max_entries * 3, device)
        self.ent_icp = _i32(max_entries, device)
        self.ent_geo = torch.zeros(max(max_entries * 4, 1), dtype=torch.float64, device=device)
        self.h = 0.0

    def struct(self) -> nat.NearLists:
        s = nat.NearLists()
        s.maxc = self.maxc
        s.cand_count = self.cand_count.data_ptr()
        s.cand_src = self.cand_src.data_ptr()
        s.excl_mask = self.excl_mask.data_ptr()
        s.hh_mask = self.hh_mask.data_ptr()
        s.max_entries = self.max_entries
        s.n_entries = self.n_entries.data_ptr()
        s.ent_tsj = self.ent_tsj.data_ptr()
        s.ent_icp = self.ent_icp.data_ptr()
        s.ent_geo = self.ent_geo.data_ptr()
        return s

    # -- builders ---------------------------------------------------------------
    @classmethod
    def build_py(cls, Xv, N, Xupv=None, thresh=0.0, maxc=32):
        """naiveNearZoneInfo on device layouts (threshold 1/N by default)."""
        nv = Xv.shape[0]
        ctx = nat.context(N, Xv.device)
        while True:
            nz = cls("py_hh", N, ctx.Nup, nv, maxc, 0, Xv.device)
            ws = ctx.workspace(ctx.lib.ves_near_zone_workspace(ctx.handle, nv))
            st = nz.struct()
            rc = ctx.lib.ves_near_zone_py(ctx.handle, nv, Xv.data_ptr(), nat.ptr(Xupv), float(thresh),
                                          ctypes.byref(st), ws.data_ptr(), ws.numel(), nat.stream_ptr(Xv.device))
            need = ctx.max_candidates()
            if rc == nat.VES_ERR_NEARLIST_OVERFLOW and need > maxc:
                maxc = nat.grow_capacity(need, maxc)
                continue
            nat.check(rc, "naiveNearZoneInfo")
            return nz

    @classmethod
    def build_matlab(cls, Xv, N, h=0.0, maxc=32, max_entries=None):
        nv = Xv.shape[0]
        ctx = nat.context(N, Xv.device)
        max_entries = max_entries or max(1024, nv * N // 4)
        while True:
            nz = cls("matlab", N, ctx.Nup, nv, maxc, max_entries, Xv.device)
            ws = ctx.workspace(ctx.lib.ves_near_zone_workspace(ctx.handle, nv))
            st = nz.struct()
            rc = ctx.lib.ves_near_zone_matlab(ctx.handle, nv, Xv.data_ptr(), float(h), ctypes.byref(st),
                                              ws.data_ptr(), ws.numel(), nat.stream_ptr(Xv.device))
            if rc == nat.VES_ERR_NEARLIST_OVERFLOW:
                need = ctx.max_candidates()
                if need > maxc:  # the candidate search stops before the entries are made
                    maxc = nat.grow_capacity(need, maxc)
                    continue
                ne = int(nz.n_entries[0].item())
                if ne > max_entries:
                    max_entries = ne + 64
                    continue
                nat.check(rc, "getZone")
            nat.check(rc, "getZone")
            if h <= 0:
                geo = torch.empty(3, nv, dtype=torch.float64, device=Xv.device)
                nat.check(ctx.lib.ves_geom_prop(ctx.handle, nv, Xv.data_ptr(), geo[0].data_ptr(), geo[1].data_ptr(),
                                                geo[2].data_ptr(), nat.stream_ptr(Xv.device)))
                h = float(geo[2].min().item()) / N
            nz.h = h
            return nz

    # -- host views in the reference's index format -------------------------------
    def _host(self):
        wN, wU = (self.N + 31) // 32, (self.Nup + 31) // 32
        cnt = self.cand_count.cpu().numpy()[: self.nv]
        src = self.cand_src.cpu().numpy()[: self.nv * self.maxc].reshape(self.nv, self.maxc)
        em = self.excl_mask.cpu().numpy().view(np.uint32)[: self.nv * self.maxc * wN].reshape(self.nv, self.maxc, wN)
        hm = self.hh_mask.cpu().numpy().view(np.uint32)[: self.nv * self.maxc * wU].reshape(self.nv, self.maxc, wU)
        return cnt, src, em, hm

    @staticmethod
    def _bits(words, n):
        b = ((words[:, None] >> np.arange(32, dtype=np.uint32)[None, :]) & 1).reshape(-1)[:n]
        return np.nonzero(b)[0]

    def ids(self):
        """(ids0, ids1, ids2): (relative source index, target point, target vesicle)."""
        cnt, src, em, _ = self._host()
        rows = []
        for t in range(self.nv):
            for c in range(cnt[t]):
                s = src[t, c]
                for i in self._bits(em[t, c], self.N):
                    rows.append((t, i, s))
        rows.sort()
        a = np.array(rows, dtype=np.int64).reshape(-1, 3)
        t, i, s = a[:, 0], a[:, 1], a[:, 2]
        return s - (t <= s).astype(np.int64), i, t

    def pairs(self):
        ids0, ids1, ids2 = self.ids()
        s = ids0 + (ids2 <= ids0).astype(np.int64)
        return ids2 * self.N + ids1, s

    def hh(self):
        """(id1_hh, id2_hh) = (s*Nup + u, t)."""
        cnt, src, _, hm = self._host()
        rows = []
        for t in range(self.nv):
            for c in range(cnt[t]):
                s = src[t, c]
                for u in self._bits(hm[t, c], self.Nup):
                    rows.append((t, s * self.Nup + u))
        rows.sort()
        a = np.array(rows, dtype=np.int64).reshape(-1, 2)
        return a[:, 1], a[:, 0]

    def __getitem__(self, k):
        if k in (4, -1):
            return self.ids()
        if k == 3:
            return self.hh()
        if k == 2:
            return self.pairs()
        raise IndexError("closest_dist / idx_closest are not materialised (O(nv^2 Nup)); "
                         "the near-singular kernel computes what it needs")

    def __len__(self):
        return 5


def naiveNearZoneInfo(vesicleX, vesicleUpX=None, max_layer_dist=None):
    """biem_support.py:520-613 (threshold ``max_layer_dist`` or 1/N)."""
    X = as_device_f64(vesicleX)
    N = X.shape[0] // 2
    Xup = None if vesicleUpX is None else to_vm(as_device_f64(vesicleUpX))
    return NearZone.build_py(to_vm(X), N, Xup, 0.0 if max_layer_dist is None else float(max_layer_dist))


def _density(sa, f, ns, dev):
    fv = to_vm(as_device_f64(f))
    sav = to_vm(as_device_f64(sa))
    nv = fv.shape[0]
    den = torch.empty_like(fv)
    nat.check(nat.load_library().ves_density(nv, ns, fv.data_ptr(), sav.data_ptr(), den.data_ptr(),
                                             nat.stream_ptr(dev)), "density")
    return den


def _exclusions_from_ids(ids, nt, Ntar, offset, nsrc, device):
    """Host conversion of (ids0, ids1, ids2) into per-column sorted candidate masks."""
    ids0, ids1, ids2 = [np.asarray(torch.as_tensor(a).cpu(), dtype=np.int64) for a in ids]
    wN = (Ntar + 31) // 32
    per = {}
    for j, i, t in zip(ids0, ids1, ids2):
        selfv = offset + t
        s = j + (1 if j >= selfv else 0)
        per.setdefault(int(t), {}).setdefault(int(s), set()).add(int(i))
    maxc = max([len(v) for v in per.values()] + [1])
    cnt = np.zeros(nt, np.int32)
    src = np.zeros((nt, maxc), np.int32)
    mask = np.zeros((nt, maxc, wN), np.uint32)
    for t, d in per.items():
        for c, s in enumerate(sorted(d)):
            src[t, c] = s
            for i in d[s]:
                mask[t, c, i >> 5] |= np.uint32(1) << np.uint32(i & 31)
        cnt[t] = len(d)
    nz = NearZone("py_hh", Ntar, Ntar, nt, maxc, 0, device)
    nz.cand_count = torch.from_numpy(cnt).to(device)
    nz.cand_src = torch.from_numpy(src.reshape(-1)).to(device)
    nz.excl_mask = torch.from_numpy(mask.reshape(-1).view(np.int32)).to(device)
    return nz


def _farfield(precision, Xsrc_v, den_v, Xtar_v, self_idx, nz, Ntar):
    dev = Xsrc_v.device
    nsrc, ns = Xsrc_v.shape[0], Xsrc_v.shape[1] // 2
    nt = Xtar_v.shape[0]
    # the near lists are laid out for N = Ntar; without them any context serves
    ctx = nat.context(Ntar if nz is not None else 16, dev)
    out = torch.empty(nt, 2 * Ntar, dtype=torch.float64, device=dev)
    prec = nat.PREC[precision]
    ws = ctx.workspace(ctx.lib.ves_farfield_workspace(ctx.handle, prec, nsrc, ns, nt, Ntar))
    st = nz.struct() if nz is not None else None
    nat.check(ctx.lib.ves_farfield(ctx.handle, prec, nsrc, ns, Xsrc_v.data_ptr(), den_v.data_ptr(), nt, Ntar,
                                   Xtar_v.data_ptr(), nat.ptr(self_idx), ctypes.byref(st) if st is not None else None,
                                   out.data_ptr(), ws.data_ptr(), ws.numel(), nat.stream_ptr(dev)), "farfield")
    return out


def allExactStokesSLTarget_compare2(vesicleX, vesicle_sa, f, tarX, ids0, ids1, ids2, length: float = 1.0,
                                    offset: int = 0, precision: str = "fp64"):
    """Far field of all other vesicles with the given near-pair exclusions
    (biem_support.py:124-228).  Target column t is vesicle ``offset + t``."""
    Xs = as_device_f64(vesicleX)
    dev = Xs.device
    ns, nsrc = Xs.shape[0] // 2, Xs.shape[1]
    tarX = as_device_f64(tarX)
    if tarX.dim() == 1:
        tarX = tarX.unsqueeze(1)
    Ntar, nt = tarX.shape[0] // 2, tarX.shape[1]
    den = _density(vesicle_sa, f, ns, dev)
    nz = _exclusions_from_ids((ids0, ids1, ids2), nt, Ntar, offset, nsrc, dev) if len(ids0) else None
    self_idx = torch.arange(offset, offset + nt, dtype=torch.int32, device=dev)
    out = _farfield(precision, to_vm(Xs), den, to_vm(tarX), self_idx, nz, Ntar)
    return from_vm(out)


def allExactStokesSLTarget_compare1(vesicleX, vesicle_sa, f, tarX, length: float = 1.0, offset: int = 0,
                                    precision: str = "fp64"):
    """Far field with exclusions computed from the (length/Ntar) rule
    (biem_support.py:7-121).  Returns (far field, (ids0, ids1, ids2))."""
    Xs = as_device_f64(vesicleX)
    dev = Xs.device
    tarX = as_device_f64(tarX)
    if tarX.dim() == 1:
        tarX = tarX.unsqueeze(1)
    Ntar, nt = tarX.shape[0] // 2, tarX.shape[1]
    ns, nsrc = Xs.shape[0] // 2, Xs.shape[1]
    ctx = nat.context(Ntar, dev)
    if ns != ctx.Nup or nt + offset > nsrc:
        raise ValueError("compare1: sources must be the Nup-upsampled vesicles of the targets")
    # exclusions: targets column t vs all sources; build on the full suspension
    # then keep the requested target columns
    tar_full = torch.zeros(2 * Ntar, nsrc, dtype=torch.float64, device=dev)
    tar_full[:, offset:offset + nt] = tarX
    nz = NearZone.build_py(to_vm(tar_full), Ntar, to_vm(Xs), float(length) / Ntar)
    ids0, ids1, ids2 = nz.ids()
    keep = (ids2 >= offset) & (ids2 < offset + nt)
    # compare1 lists (relative source, target point, target column) in that
    # lexicographic order (torch.where over (nv-1, Ntar*ntar), :72-75)
    order = np.lexsort((ids2[keep], ids1[keep], ids0[keep]))
    ids = (ids0[keep][order], ids1[keep][order], ids2[keep][order] - offset)
    far = allExactStokesSLTarget_compare2(vesicleX, vesicle_sa, f, tarX, *ids, length=length, offset=offset,
                                          precision=precision)
    return far, (ids[0], ids[1], ids[2] + offset)


def wrapper_allExactStokesSLTarget_compare2(vesicleX, vesicle_sa, fup, tarX, info_stokes, precision: str = "fp64"):
    """biem_support.py:231-272 (target chunking is unnecessary on the device)."""
    return allExactStokesSLTarget_compare2(vesicleX, vesicle_sa, fup, tarX, *info_stokes, precision=precision)


def exactStokesSL_(vesicle, f, Xtar=None, K1=None, precision: str = "fp64"):
    """Single layer of the vesicles ``K1`` of ``vesicle`` at every column of
    ``Xtar`` (biem_support.py:334-389, evaluated per target column)."""
    Xtar = as_device_f64(Xtar)
    K1 = list(range(vesicle.nv)) if K1 is None else list(K1)
    dev = Xtar.device
    N = vesicle.N
    Xs = vesicle.X[:, K1]
    den = _density(vesicle.sa[:, K1], as_device_f64(f)[:, K1], N, dev)
    Ntar, nc = Xtar.shape[0] // 2, Xtar.shape[1]
    out = _farfield(precision, to_vm(Xs), den, to_vm(Xtar), None, None, Ntar)
    return from_vm(out)


def upsample_factor(N: int) -> int:
    """Nup = N * ceil(sqrt(N)) (poten.py:24)."""
    return N * math.ceil(math.sqrt(N))
