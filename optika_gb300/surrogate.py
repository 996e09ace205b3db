"""Learned surrogate of a batched trace's ray map, trained and run on the
tensor cores, with the plain trace as its fallback and its accuracy reference.

The reference has no counterpart: this is the learned part built on top of
the batched spectrograph trace (``optika_gb300.batch``).  For every ray of a
configuration the surrogate maps 9 inputs -- field x, y, pupil x, y and
wavelength, each normalised to [-1, 1], plus 4 normalised configuration
parameters -- through an MLP (4 hidden layers of 256, SiLU, BF16 weights and
activations, FP32 accumulation) to 3 outputs: the image position's residual
over a per-configuration quadratic polynomial of the 5 ray inputs (in units
of ``out_scale`` mm) and a vignetting logit.

Everything runs in this package's own kernels through the C-ABI:
``otx_surrogate_pack`` builds the inputs from the device-generated batch
rays (no input traffic), ``otx_gemm_bf16`` (TMA + tcgen05 + TMEM) runs every
layer forward and backward, ``otx_surrogate_loss`` forms the loss gradient,
``otx_colsum_bf16`` the bias gradients and ``otx_adam`` the update.
``otx_surrogate_image`` simulates sensor images: rays of trusted
configurations whose logit is at least ``logit_band`` from 0 land at the
predicted position; all other rays are traced by the plain kernel inside the
same launch.  The baseline polynomial is fitted by least squares (float64,
on the device) from the training rays.
"""

from __future__ import annotations

import ctypes
import itertools
import math
import time
from typing import Sequence

import numpy as np
import torch

from . import _lib as L
from ._api import device, ptr, stream_handle

HIDDEN = (256, 256, 256, 256)


def config_features(params: np.ndarray) -> np.ndarray:
    """Normalised configuration inputs of the spectrograph batch:
    (1/d0 - 2400)/200, a1/1e-4, a2/1e-7, tilt/2 deg."""
    p = np.asarray(params, dtype=np.float64)
    return np.stack([(1.0 / p[:, 0] - 2400.0) / 200.0, p[:, 1] / 1e-4, p[:, 2] / 1e-7,
                     p[:, 3] / (2.0 * math.pi / 180.0)], axis=-1).astype(np.float32)


def quadratic_basis(u: torch.Tensor) -> torch.Tensor:
    """Terms 1, u_i, u_i u_j (i <= j) of 5 inputs, in the kernel's order."""
    cols = [torch.ones_like(u[:, 0])] + [u[:, i] for i in range(5)]
    cols += [u[:, i] * u[:, j] for i, j in itertools.combinations_with_replacement(range(5), 2)]
    return torch.stack(cols, dim=-1)


class MLP:
    """The surrogate's network on the tensor-core kernels.

    Weights are kept as FP32 masters (updated by Adam) with BF16 copies in
    both orientations: ``w16[l]`` [out x in] is the forward GEMM's B operand,
    ``w16t[l]`` [in x out] the backward one's.  Row pitches are multiples of
    8 elements (16 bytes), as the TMA tensor maps need.
    """

    def __init__(self, widths: Sequence[int], seed: int, dev: torch.device):
        self.widths = tuple(int(w) for w in widths)
        self.dev = dev
        self.lib = L.load()
        g = torch.Generator().manual_seed(seed)
        self.w, self.b, self.w16, self.w16t = [], [], [], []
        self.m = []
        self.v = []
        n_layers = len(self.widths) - 1
        for l in range(n_layers):
            fin, fout = self.widths[l], self.widths[l + 1]
            std = math.sqrt(2.0 / fin) if l < n_layers - 1 else 0.01
            w = (torch.randn((fout, fin), generator=g) * std).to(dev)
            b = torch.zeros(fout, device=dev)
            self.w.append(w)
            self.b.append(b)
            self.w16.append(torch.zeros((fout, _pad8(fin)), dtype=torch.bfloat16, device=dev))
            self.w16t.append(torch.zeros((fin, _pad8(fout)), dtype=torch.bfloat16, device=dev))
            self.m.append([torch.zeros_like(w), torch.zeros_like(b)])
            self.v.append([torch.zeros_like(w), torch.zeros_like(b)])
        self.step_count = 0
        self.err = torch.zeros(1, dtype=torch.int32, device=dev)
        self.gw = [torch.zeros_like(w) for w in self.w]
        self.gb = [torch.zeros_like(b) for b in self.b]
        self._bufs = {}
        self.refresh_bf16()

    # -- parameters ------------------------------------------------------
    def refresh_bf16(self) -> None:
        """BF16 copies from the FP32 masters (an Adam step with zero rate)."""
        for l in range(len(self.w)):
            w = self.w[l]
            zero = torch.zeros_like(w)
            st = self.lib.otx_adam(ptr(w), ptr(zero), ptr(zero.clone()), ptr(zero), w.shape[0],
                                   w.shape[1], 0.0, 0.0, 0.0, 1.0, 1, ptr(self.w16[l]),
                                   self.w16[l].shape[1], ptr(self.w16t[l]), self.w16t[l].shape[1],
                                   stream_handle())
            L.check(st, "otx_adam")

    def state_dict(self) -> dict:
        return {"widths": self.widths, "w": [t.cpu() for t in self.w],
                "b": [t.cpu() for t in self.b], "m": [[a.cpu(), b.cpu()] for a, b in self.m],
                "v": [[a.cpu(), b.cpu()] for a, b in self.v], "step": self.step_count}

    def load_state_dict(self, sd: dict) -> None:
        if tuple(sd["widths"]) != self.widths:
            raise ValueError("checkpoint widths differ from the network's")
        for l in range(len(self.w)):
            self.w[l].copy_(sd["w"][l])
            self.b[l].copy_(sd["b"][l])
            for j in range(2):
                self.m[l][j].copy_(sd["m"][l][j])
                self.v[l][j].copy_(sd["v"][l][j])
        self.step_count = int(sd["step"])
        self.refresh_bf16()

    # -- buffers ---------------------------------------------------------
    def buffers(self, rows: int, train: bool) -> dict:
        key = (rows, train)
        if key in self._bufs:
            return self._bufs[key]
        if rows % 8:
            raise ValueError("batch rows must be a multiple of 8 (16-byte rows of the transposes)")
        dev, bf = self.dev, torch.bfloat16
        nl = len(self.widths) - 1
        b = {"x": torch.zeros((rows, L.SURROGATE_LDX), dtype=bf, device=dev),
             "y": torch.zeros((rows, 4), dtype=torch.float32, device=dev),
             "aux": torch.zeros((rows, 4), dtype=torch.float32, device=dev)}
        if train:
            b["xt"] = torch.zeros((L.SURROGATE_LDX, rows), dtype=bf, device=dev)
            b["h"] = [torch.empty((rows, self.widths[l + 1]), dtype=bf, device=dev)
                      for l in range(nl - 1)]
            b["ht"] = [torch.empty((self.widths[l + 1], rows), dtype=bf, device=dev)
                       for l in range(nl - 1)]
            b["z"] = [torch.empty((rows, self.widths[l + 1]), dtype=bf, device=dev)
                      for l in range(nl - 1)]
            wmax = max(self.widths[1:-1])
            b["dz"] = [torch.empty((rows, wmax), dtype=bf, device=dev) for _ in range(2)]
            b["dzt"] = [torch.empty((wmax, rows), dtype=bf, device=dev) for _ in range(2)]
            b["dy"] = torch.zeros((rows, 8), dtype=bf, device=dev)
            b["dyt"] = torch.zeros((8, rows), dtype=bf, device=dev)
            b["sums"] = torch.zeros(4, dtype=torch.float32, device=dev)
        else:
            wmax = max(self.widths[1:-1])
            b["h"] = [torch.empty((rows, wmax), dtype=bf, device=dev) for _ in range(2)]
        self._bufs[key] = b
        return b

    # -- passes ----------------------------------------------------------
    def _gemm(self, a, lda, bmat, ldb, m, n, k, bias, epi, out, ldo, z=None, out_t=None, ldt=0):
        st = self.lib.otx_gemm_bf16(ptr(a), lda, ptr(bmat), ldb, m, n, k, ptr(bias), epi, ptr(out),
                                    ldo, ptr(z), ptr(out_t), ldt, ptr(self.err), stream_handle())
        L.check(st, "otx_gemm_bf16")

    def forward(self, bufs: dict, rows: int, train: bool) -> torch.Tensor:
        """y [rows x 4] (residual x, y, logit, unused) from bufs["x"]."""
        nl = len(self.widths) - 1
        src, lds = bufs["x"], L.SURROGATE_LDX
        for l in range(nl):
            fin, fout = self.widths[l], self.widths[l + 1]
            if l == nl - 1:
                self._gemm(src, lds, self.w16[l], self.w16[l].shape[1], rows, fout, fin, self.b[l],
                           L.EPI_BIAS_F32, bufs["y"], 4)
                break
            if train:
                dst = bufs["h"][l]
                self._gemm(src, lds, self.w16[l], self.w16[l].shape[1], rows, fout, fin, self.b[l],
                           L.EPI_SILU_BF16, dst, fout, z=bufs["z"][l], out_t=bufs["ht"][l],
                           ldt=rows)
            else:
                dst = bufs["h"][l % 2]
                self._gemm(src, lds, self.w16[l], self.w16[l].shape[1], rows, fout, fin, self.b[l],
                           L.EPI_SILU_BF16, dst, dst.shape[1])
            src, lds = dst, dst.shape[1]
        return bufs["y"]

    def backward(self, bufs: dict, rows: int) -> None:
        """Gradients of every weight and bias into gw, gb from bufs["dy"]."""
        nl = len(self.widths) - 1
        lib, sh = self.lib, stream_handle()
        # dW[l] = dZ_l^T H_{l-1}: A = dZ_l^T [out x rows], B = H_{l-1}^T [in x rows]
        dz, ldz, dzt = bufs["dy"], 8, bufs["dyt"]
        for l in range(nl - 1, -1, -1):
            fin, fout = self.widths[l], self.widths[l + 1]
            hin_t = bufs["xt"] if l == 0 else bufs["ht"][l - 1]
            self._gemm(dzt, rows, hin_t, rows, fout, fin, rows, None, L.EPI_F32_ATOMIC,
                       self.gw[l], fin)
            L.check(lib.otx_colsum_bf16(ptr(dz), rows, fout, ldz, ptr(self.gb[l]), sh),
                    "otx_colsum_bf16")
            if l == 0:
                break
            # dZ_{l-1} = (dZ_l W_l) * silu'(Z_{l-1}): A = dZ_l [rows x out], B = W_l^T [in x out]
            nxt, nxt_t = bufs["dz"][l % 2], bufs["dzt"][l % 2]
            self._gemm(dz, ldz, self.w16t[l], self.w16t[l].shape[1], rows, fin, fout, None,
                       L.EPI_DSILU_BF16, nxt, nxt.shape[1], z=bufs["z"][l - 1], out_t=nxt_t,
                       ldt=rows)
            dz, ldz, dzt = nxt, nxt.shape[1], nxt_t

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        self.step_count += 1
        sh = stream_handle()
        for l in range(len(self.w)):
            w, b = self.w[l], self.b[l]
            L.check(self.lib.otx_adam(ptr(w), ptr(self.m[l][0]), ptr(self.v[l][0]), ptr(self.gw[l]),
                                      w.shape[0], w.shape[1], lr, beta1, beta2, eps,
                                      self.step_count, ptr(self.w16[l]), self.w16[l].shape[1],
                                      ptr(self.w16t[l]), self.w16t[l].shape[1], sh), "otx_adam")
            L.check(self.lib.otx_adam(ptr(b), ptr(self.m[l][1]), ptr(self.v[l][1]), ptr(self.gb[l]),
                                      1, b.shape[0], lr, beta1, beta2, eps, self.step_count, None, 0,
                                      None, 0, sh), "otx_adam")

    def desc(self) -> L.Mlp:
        """The network for the fused kernels: BF16 weights, FP32 biases."""
        m = L.Mlp()
        m.num_inputs = self.widths[0]
        m.num_hidden = len(self.widths) - 2
        m.width = self.widths[1]
        m.num_outputs = self.widths[-1]
        for l in range(len(self.w)):
            m.w[l] = ptr(self.w16[l])
            m.ld[l] = self.w16[l].shape[1]
            m.b[l] = ptr(self.b[l])
        return m

    def check_errors(self) -> None:
        if int(self.err.item()) != 0:
            raise RuntimeError("a tensor-core GEMM gave up waiting for its pipeline")


def _pad8(n: int) -> int:
    return (n + 7) // 8 * 8


class RayMapSurrogate:
    """Surrogate of the batched spectrograph's ray map over a fixed set of
    configurations (``systems`` with their parameters ``params[c, 4]``:
    d0, a1, a2, tilt)."""

    def __init__(self, systems: Sequence, params: np.ndarray, *, overrides=(2, 3),
                 wavelength=(58.0, 63.0), field_half=(0.0, 0.0), pupil_half=40.0,
                 pixel=0.0135, out_scale: float = 0.005, logit_band: float = 0.5,
                 hidden=HIDDEN, seed: int = 5):
        self.dev = device()
        self.systems = list(systems)
        self.overrides = tuple(overrides)
        self.wavelength, self.field_half, self.pupil_half = wavelength, field_half, pupil_half
        self.pixel = float(pixel)
        self.seed = int(seed)
        n = len(self.systems)
        self.cin = torch.from_numpy(config_features(params)).to(self.dev)
        self.coef = torch.zeros((n, 2, L.SURROGATE_NBASE), dtype=torch.float32, device=self.dev)
        self.trusted = torch.ones(n, dtype=torch.uint8, device=self.dev)
        sg = L.Surrogate()
        sg.num_configs = n
        sg.config_inputs = ptr(self.cin)
        sg.baseline = ptr(self.coef)
        sg.trusted = ptr(self.trusted)
        sg.out_scale = float(out_scale)
        sg.logit_band = float(logit_band)
        self.sg = sg
        self.mlp = MLP((L.SURROGATE_NIN, *hidden, 3), seed, self.dev)
        self.lib = L.load()
        self.history: list[dict] = []

    # -- data ------------------------------------------------------------
    def traced(self, ray_counts, seed: int, image: bool = False,
               outputs=("px", "py", "unvignetted")):
        """A batch of these configurations with its own seed (rays generated
        on the device), traced by the plain kernel when outputs are asked."""
        from .batch import BatchedTrace

        bt = BatchedTrace(self.systems, overrides=list(self.overrides), ray_counts=ray_counts,
                          seed=seed, wavelength=self.wavelength, field_half=self.field_half,
                          pupil_half=self.pupil_half, image=image, tile_size=8192,
                          outputs=outputs)
        if outputs:
            bt.run()
        return bt

    def _pack(self, bt, first, rows, bufs, perm=None, targets=False, u=None, xt=None):
        st = self.lib.otx_surrogate_pack(
            ctypes.byref(bt.batch), ctypes.byref(self.sg), first, rows, ptr(perm),
            ptr(bt.bufs["px"]) if targets else None, ptr(bt.bufs["py"]) if targets else None,
            ptr(bt.bufs["unvignetted"]) if targets else None, ptr(bufs["x"]), ptr(xt),
            rows if xt is not None else 0, ptr(bufs["aux"]), ptr(u), stream_handle())
        L.check(st, "otx_surrogate_pack")

    # -- baseline ----------------------------------------------------------
    def fit_baseline(self, bt, max_rays_per_config: int = 400_000) -> None:
        """Least-squares quadratic of the traced image position over the 5
        normalised ray inputs, per configuration (float64 normal equations
        on the device)."""
        n = len(self.systems)
        offs = bt.ray_offset_host
        chunk = 1 << 20
        bufs = {"x": torch.empty((chunk, L.SURROGATE_LDX), dtype=torch.bfloat16, device=self.dev),
                "aux": torch.empty((chunk, 4), dtype=torch.float32, device=self.dev)}
        u = torch.empty((chunk, 8), dtype=torch.float32, device=self.dev)
        ata = torch.zeros((n, L.SURROGATE_NBASE, L.SURROGATE_NBASE), dtype=torch.float64,
                          device=self.dev)
        aty = torch.zeros((n, L.SURROGATE_NBASE, 2), dtype=torch.float64, device=self.dev)
        for c in range(n):
            lo, hi = int(offs[c]), int(offs[c + 1])
            hi = min(hi, lo + max_rays_per_config)
            for f in range(lo, hi, chunk):
                rows = min(chunk, hi - f)
                self._pack(bt, f, rows, bufs, u=u)
                m = bt.bufs["unvignetted"][f:f + rows].bool()
                F = quadratic_basis(u[:rows, :5][m].double())
                y = torch.stack([bt.bufs["px"][f:f + rows][m], bt.bufs["py"][f:f + rows][m]],
                                -1).double()
                ata[c] += F.T @ F
                aty[c] += F.T @ y
        # the normal equations (one 21 x 21 system per configuration) are
        # accumulated on the device and solved on the host: set-up, not
        # the traced or simulated rays
        reg = 1e-9 * torch.eye(L.SURROGATE_NBASE, dtype=torch.float64)
        sol = torch.linalg.solve(ata.cpu() + reg, aty.cpu())  # [n, NBASE, 2]
        self.coef.copy_(sol.permute(0, 2, 1).float())

    # -- training ----------------------------------------------------------
    def train(self, bt, steps: int, batch: int = 65536, lr: float = 1e-3, lr_min: float = 1e-5,
              warmup: int = 100, w_pos: float = 1.0, w_cls: float = 1.0,
              log_every: int = 200) -> list[dict]:
        """Adam on random batches of the traced rays, cosine-decayed rate."""
        bufs = self.mlp.buffers(batch, train=True)
        total = bt.total
        perm = torch.randperm(total, device=self.dev)
        pos = 0
        lib, sh = self.lib, stream_handle()
        t0 = time.perf_counter()
        bufs["sums"].zero_()
        for step in range(steps):
            if pos + batch > total:
                perm = torch.randperm(total, device=self.dev)
                pos = 0
            self._pack(bt, pos, batch, bufs, perm=perm, targets=True, xt=bufs["xt"])
            pos += batch
            self.mlp.forward(bufs, batch, train=True)
            st = lib.otx_surrogate_loss(ptr(bufs["y"]), 4, ptr(bufs["aux"]), batch, w_pos, w_cls,
                                        1.0 / batch, ptr(bufs["dy"]), ptr(bufs["dyt"]), batch,
                                        ptr(bufs["sums"]), sh)
            L.check(st, "otx_surrogate_loss")
            self.mlp.backward(bufs, batch)
            if step < warmup:
                rate = lr * (step + 1) / warmup
            else:
                p = (step - warmup) / max(1, steps - warmup)
                rate = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * p))
            self.mlp.adam(rate)
            if (step + 1) % log_every == 0 or step == steps - 1:
                s = bufs["sums"].tolist()
                k = log_every if (step + 1) % log_every == 0 else (step + 1) % log_every
                n_lab = max(s[2], 1.0)
                rec = {"step": step + 1, "lr": rate,
                       "rms_residual_px": math.sqrt(s[0] / n_lab) * self.sg.out_scale / self.pixel
                       / math.sqrt(2.0),
                       "bce": s[1] / (k * batch), "accuracy": s[3] / (k * batch),
                       "seconds": time.perf_counter() - t0}
                self.history.append(rec)
                bufs["sums"].zero_()
        self.mlp.check_errors()
        return self.history

    # -- inference -----------------------------------------------------------
    def predict(self, bt, chunk: int = 131072, fused: bool = True):
        """Network outputs for every ray of a batch: predicted positions (mm,
        sensor frame), logits, and the baseline positions.  ``fused``: the
        positions and logits come from the fused image kernel (the one that
        simulates images), the baseline from the packing kernel; otherwise
        everything from the layer-by-layer path."""
        if fused:
            return self._predict_fused(bt, chunk)
        total = bt.total
        px = torch.empty(total, device=self.dev)
        py = torch.empty(total, device=self.dev)
        logit = torch.empty(total, device=self.dev)
        bx = torch.empty(total, device=self.dev)
        by = torch.empty(total, device=self.dev)
        bufs = self.mlp.buffers(chunk, train=False)
        s = self.sg.out_scale
        for f in range(0, total, chunk):
            rows = min(chunk, total - f)
            self._pack(bt, f, rows, bufs)
            y = self.mlp.forward(bufs, rows, train=False)
            aux = bufs["aux"]
            px[f:f + rows] = aux[:rows, 0] + s * y[:rows, 0]
            py[f:f + rows] = aux[:rows, 1] + s * y[:rows, 1]
            logit[f:f + rows] = y[:rows, 2]
            bx[f:f + rows] = aux[:rows, 0]
            by[f:f + rows] = aux[:rows, 1]
        self.mlp.check_errors()
        return {"px": px, "py": py, "logit": logit, "base_x": bx, "base_y": by}

    def _predict_fused(self, bt, chunk: int):
        total = bt.total
        out = torch.empty((total, 4), device=self.dev)
        base = torch.empty((total, 2), device=self.dev)
        bufs = self.mlp.buffers(chunk, train=False)
        for f in range(0, total, chunk):
            rows = min(chunk, total - f)
            self._pack(bt, f, rows, bufs)
            base[f:f + rows] = bufs["aux"][:rows, :2]
        stats = torch.zeros(4, dtype=torch.int64, device=self.dev)
        net = self.mlp.desc()
        need = int(self.lib.otx_surrogate_image_fused_workspace(ctypes.byref(bt.batch),
                                                                ctypes.byref(net), total))
        ws = torch.empty(max(need, 256), dtype=torch.uint8, device=self.dev)
        st = self.lib.otx_surrogate_image_fused(
            ctypes.byref(bt.lowering.sys), ctypes.byref(bt.batch), ctypes.byref(self.sg),
            ctypes.byref(net), 0, total, None, ptr(out), ptr(ws), need, ptr(stats),
            ptr(self.mlp.err), stream_handle())
        L.check(st, "otx_surrogate_image_fused")
        self.mlp.check_errors()
        return {"px": out[:, 0], "py": out[:, 1], "logit": out[:, 2], "base_x": base[:, 0],
                "base_y": base[:, 1]}

    def evaluate(self, bt_eval, budget_px: float = 0.05) -> dict:
        """Errors against the plain trace of a held-out batch (already run).

        Rays the surrogate lands (trusted configuration, |logit| >= band,
        logit > 0) are compared with the traced position; rays it routes to
        the trace carry no error.  Returns per-configuration and overall RMS
        and 99.9th-percentile errors (px), the fallback fraction, the
        relative efficiency (landed flux) error, and the baseline-only
        error for comparison."""
        pred = self.predict(bt_eval)
        tx, ty = bt_eval.bufs["px"], bt_eval.bufs["py"]
        lab = bt_eval.bufs["unvignetted"].bool()
        cfg = torch.repeat_interleave(torch.arange(len(self.systems), device=self.dev),
                                      torch.from_numpy(bt_eval.counts).to(self.dev))
        band = self.sg.logit_band
        trusted = self.trusted.bool()[cfg]
        routed = trusted & (pred["logit"].abs() >= band)
        fallback = ~routed
        land = routed & (pred["logit"] > 0)
        both = land & lab
        err = torch.hypot(pred["px"] - tx, pred["py"] - ty) / self.pixel
        base_err = torch.hypot(pred["base_x"] - tx, pred["base_y"] - ty) / self.pixel
        e = err[both]
        eb = base_err[lab]
        n_true = int(lab.sum())
        n_landed = int(land.sum()) + int((fallback & lab).sum())
        out = {
            "rays": int(bt_eval.total),
            "rms_px": float(e.square().mean().sqrt()) if e.numel() else 0.0,
            "p999_px": float(torch.quantile(e[:1 << 24].float(), 0.999)) if e.numel() else 0.0,
            "max_px": float(e.max()) if e.numel() else 0.0,
            "baseline_rms_px": float(eb.square().mean().sqrt()),
            "baseline_p999_px": float(torch.quantile(eb[:1 << 24].float(), 0.999)),
            "fallback_fraction": float(fallback.float().mean()),
            "false_pass": int((land & ~lab).sum()),
            "false_block": int((routed & ~(pred["logit"] > 0) & lab).sum()),
            "efficiency_rel_error": abs(n_landed - n_true) / max(n_true, 1),
            "budget_px": budget_px,
        }
        per = []
        for c in range(len(self.systems)):
            m = both & (cfg == c)
            ec = err[m]
            per.append(float(ec.square().mean().sqrt()) if ec.numel() else 0.0)
        out["per_config_rms_px"] = per
        return out

    def set_trust(self, per_config_rms_px: Sequence[float], budget_px: float) -> int:
        """Configurations whose held-out RMS exceeds the budget are routed
        entirely to the trace; returns how many stay trusted."""
        t = torch.tensor([1 if r <= budget_px else 0 for r in per_config_rms_px],
                         dtype=torch.uint8, device=self.dev)
        self.trusted.copy_(t)
        return int(t.sum())

    def image(self, bt, chunk: int | None = None, fused: bool = True):
        """Sensor images of a batch (bt built with image=True): network for
        confidently classified rays of trusted configurations, plain trace
        for the rest.  Returns (images, stats[4] = rays, traced, binned by
        the network, binned by the trace).

        ``fused`` (default): one persistent tensor-core kernel per call of
        up to ``chunk`` rays (default 2**28) generates the rays, runs the
        whole network on chip and bins, and a second kernel traces the rays
        it queued (``otx_surrogate_image_fused``).  Otherwise the network
        runs layer by layer (``otx_gemm_bf16``) over chunks of ``chunk``
        rays (default 131072) with the activations in HBM."""
        if bt.images is None:
            raise ValueError("the batch needs image=True")
        bt.images.zero_()
        stats = torch.zeros(4, dtype=torch.int64, device=self.dev)
        lib, sh = self.lib, stream_handle()
        total = bt.total
        if fused:
            chunk = chunk or (1 << 28)
            net = self.mlp.desc()
            for f in range(0, total, chunk):
                rows = min(chunk, total - f)
                need = int(lib.otx_surrogate_image_fused_workspace(ctypes.byref(bt.batch),
                                                                   ctypes.byref(net), rows))
                ws = torch.empty(max(need, 256), dtype=torch.uint8, device=self.dev)
                st = lib.otx_surrogate_image_fused(
                    ctypes.byref(bt.lowering.sys), ctypes.byref(bt.batch), ctypes.byref(self.sg),
                    ctypes.byref(net), f, rows, ctypes.byref(bt.img), None, ptr(ws), need,
                    ptr(stats), ptr(self.mlp.err), sh)
                L.check(st, "otx_surrogate_image_fused")
            return bt.images, stats
        chunk = chunk or 131072
        bufs = self.mlp.buffers(chunk, train=False)
        for f in range(0, total, chunk):
            rows = min(chunk, total - f)
            self._pack(bt, f, rows, bufs)
            self.mlp.forward(bufs, rows, train=False)
            st = lib.otx_surrogate_image(ctypes.byref(bt.lowering.sys), ctypes.byref(bt.batch),
                                         ctypes.byref(self.sg), f, rows, ptr(bufs["y"]), 4,
                                         ptr(bufs["aux"]), ctypes.byref(bt.img), ptr(stats), sh)
            L.check(st, "otx_surrogate_image")
        return bt.images, stats

    def save(self, path) -> None:
        torch.save({"mlp": self.mlp.state_dict(), "coef": self.coef.cpu(),
                    "trusted": self.trusted.cpu(), "out_scale": self.sg.out_scale,
                    "logit_band": self.sg.logit_band}, path)

    def load(self, path) -> None:
        sd = torch.load(path, map_location="cpu")
        self.mlp.load_state_dict(sd["mlp"])
        self.coef.copy_(sd["coef"])
        self.trusted.copy_(sd["trusted"])
        self.sg.out_scale = float(sd["out_scale"])
        self.sg.logit_band = float(sd["logit_band"])
