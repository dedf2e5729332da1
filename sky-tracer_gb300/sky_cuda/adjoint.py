"""Differentiable sky rendering: the forward/backward pair of the C ABI
(sky_cuda_adjoint_forward / sky_cuda_adjoint_backward) and a
torch.autograd.Function over it.

No counterpart in the reference, which renders a fixed medium.  The medium
of a differentiable render is the scene's with parameters applied (see
include/sky_cuda.h): per majorant layer, density scales of Rayleigh, Mie
(aerosol species 0) and ozone; the Mie single-scattering albedo and
Henyey-Greenstein g; optionally per band, multipliers of the Rayleigh, Mie
and ozone cross sections and of the solar radiance.  Gradients come from
path-replay backpropagation on the GPU: no path is stored.

    r = AdjointRenderer(gpu_scene, RenderConfig(width=128, height=64, spp=64))
    theta = torch.tensor(initial_layer_params(scene, g=0.76), device="cuda", requires_grad=True)
    film = render_film(r, theta)                 # [H, W, B], differentiable
    loss = ((film_to_xyz(film, scene) - target) ** 2).sum()
    loss.backward()                              # theta.grad via the adjoint kernel
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import SkyAdjointGrads, SkyAdjointJob, SkyAdjointParams, SkyDeviceOutputs, check
from .render import GpuScene, RenderConfig
from .scene import Scene

BAND_PARAMS = _abi.ADJOINT_BAND_PARAMS
PARAMS_PER_LAYER = 3  # Rayleigh, Mie, ozone density scales
SEGMENT_INTEGRALS = _abi.ADJOINT_SEGMENT_INTEGRALS  # default backward estimator (lower variance)
NULL_COLLISIONS = _abi.ADJOINT_NULL_COLLISIONS      # exact derivative of the forward estimator
DECORRELATE_SEED = 0x9E3779B97F4A7C15  # xor-ed into the seed of a decorrelated backward pass


def mie_albedo(scene: Scene) -> float:
    """Single-scattering albedo of aerosol species 0, averaged over bands."""
    o = scene.aerosol_optics.reshape(scene.band_count, _abi.SPECIES_COUNT)[:, 0]
    sca = o["scattering_km_inv_per_g_m3"].astype(np.float64)
    ext = sca + o["absorption_km_inv_per_g_m3"].astype(np.float64)
    keep = ext > 0
    return float(np.mean(sca[keep] / ext[keep])) if keep.any() else 0.0


def initial_layer_params(scene: Scene, g: float) -> np.ndarray:
    """Parameters that reproduce `scene` (scales 1, the scene's Mie albedo, HG g)."""
    layers = scene.layer_count
    p = np.ones(PARAMS_PER_LAYER * layers + 2, dtype=np.float32)
    p[PARAMS_PER_LAYER * layers] = mie_albedo(scene)
    p[PARAMS_PER_LAYER * layers + 1] = g
    return p


def param_names(layers: int) -> list[str]:
    names = [f"{kind}[{l}]" for l in range(layers) for kind in ("rayleigh", "mie", "ozone")]
    return names + ["mie_albedo", "mie_g"]


def fd_check_parameters(grad, layers: int, count: int = 16, seed: int = 4, floor: float = 1e-4) -> list[int]:
    """Indices of `count` parameters for a finite-difference check of a
    gradient: the Mie albedo and g always, the others drawn with `seed`
    evenly from the Rayleigh, Mie and ozone layer scales whose gradient is
    at least `floor` times the largest (a layer without the species, such as
    ozone outside its tent, has a zero gradient and checks nothing)."""
    g = np.abs(np.asarray(grad, dtype=np.float64))
    top = float(g.max()) if g.size else 0.0
    rng = np.random.default_rng(seed)
    picked = [PARAMS_PER_LAYER * layers, PARAMS_PER_LAYER * layers + 1]
    pools = [[PARAMS_PER_LAYER * l + k for l in range(layers) if g[PARAMS_PER_LAYER * l + k] >= floor * top]
             for k in range(PARAMS_PER_LAYER)]
    want = count - len(picked)
    for k, pool in enumerate(pools):
        n = min(len(pool), want // PARAMS_PER_LAYER + (1 if k < want % PARAMS_PER_LAYER else 0))
        picked += [int(i) for i in rng.choice(pool, n, replace=False)] if n else []
    spare = [i for pool in pools for i in pool if i not in picked]
    if len(picked) < count and spare:
        picked += [int(i) for i in rng.choice(spare, min(count - len(picked), len(spare)), replace=False)]
    return sorted(picked)


def _ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


class AdjointRenderer:
    """Forward and backward renders of one RenderConfig on a GpuScene.

    Tensors are CUDA torch tensors; calls are queued on torch's current
    stream.  Tracking defaults to merged layers (the fastest mode)."""

    def __init__(self, gs: GpuScene, config: RenderConfig, estimator: int = SEGMENT_INTEGRALS):
        import torch
        if config.tracking == _abi.TRACKING_SEGMENT_RESTART:
            config = RenderConfig(**{**config.__dict__, "tracking": _abi.TRACKING_MERGED_LAYERS})
        self.gs = gs
        self.lib = gs.lib
        self.config = config
        self.estimator = estimator
        self._c_config = config.to_c()
        self.bands = gs.band_count
        self.pixels = config.pixels
        self.param_count = int(self.lib.sky_cuda_adjoint_param_count(gs.handle))
        self.layers = (self.param_count - 2) // PARAMS_PER_LAYER
        self._status = torch.zeros(1, dtype=torch.int32, device="cuda")
        # render_film's forward and backward wait for the GPU and read the watchdog
        # status after every call; a caller that queues many calls (one per sun
        # elevation, say) sets this to False and calls check_status() once after them
        self.check_each_call = True

    @property
    def chain_count(self) -> int:
        """Chains of one render: the length of a chain-radiance buffer."""
        return self.pixels * self.bands * self.config.spp

    def new_chain_buffer(self):
        """A chain-radiance buffer for forward(chains=...) / backward(chains=...)."""
        import torch
        return torch.empty(self.chain_count, dtype=torch.float32, device="cuda")

    def _params(self, layer, band, sample_layer=None, sample_band=None, sun=None, chains=None) -> SkyAdjointParams:
        for name, t, n in (("layer_params", layer, self.param_count), ("sample_layer_params", sample_layer,
                                                                       self.param_count),
                           ("band_params", band, self.bands * BAND_PARAMS),
                           ("sample_band_params", sample_band, self.bands * BAND_PARAMS)):
            if t is None:
                continue
            if not (t.is_cuda and t.is_contiguous()) or t.numel() != n or str(t.dtype) != "torch.float32":
                raise ValueError(f"{name} must be a contiguous float32 CUDA tensor of {n} values")
        p = SkyAdjointParams()
        p.layer_params = _ptr(layer)
        p.band_params = _ptr(band)
        p.sample_layer_params = _ptr(sample_layer)
        p.sample_band_params = _ptr(sample_band)
        p.sun_direction = (ctypes.c_float * 3)(*(sun if sun is not None else (0.0, 0.0, 0.0)))
        p.estimator = self.estimator
        if chains is not None:
            if not (chains.is_cuda and chains.is_contiguous()) or chains.numel() != self.chain_count or \
                    str(chains.dtype) != "torch.float32":
                raise ValueError(f"chains must be a contiguous float32 CUDA tensor of {self.chain_count} values")
            p.chain_radiance = chains.data_ptr()
            p.chain_radiance_len = chains.numel()
        return p

    def check_status(self) -> None:
        """Wait for the queued calls and raise RenderWatchdog if any of them
        tripped the path watchdog since the last check."""
        self._check_status()

    def _check_status(self) -> None:
        import torch
        torch.cuda.current_stream().synchronize()
        if int(self._status.item()):
            self._status.zero_()
            raise _abi.RenderWatchdog(_abi.SKY_ERR_WATCHDOG, "GPU path watchdog was reached")

    def forward(self, layer, band=None, *, sample_layer=None, sample_band=None, sun=None, xyz: bool = False,
                check_status: bool = True, chains=None) -> dict:
        """Film [pixels * B] (float32) and cell sums; XYZ and its variance too with xyz=True.
        chains (new_chain_buffer()) receives every chain's radiance for a
        backward at the same parameters and sun."""
        import torch
        cells = self.pixels * self.bands
        out = {
            "cell_sum": torch.empty(cells, dtype=torch.float64, device="cuda"),
            "cell_sumsq": torch.empty(cells, dtype=torch.float64, device="cuda"),
            "film": torch.empty(cells, dtype=torch.float32, device="cuda"),
        }
        if xyz:
            out["xyz"] = torch.empty(self.pixels * 3, dtype=torch.float64, device="cuda")
            out["xyz_var"] = torch.empty(self.pixels * 3, dtype=torch.float64, device="cuda")
        o = SkyDeviceOutputs()
        for name, _ in SkyDeviceOutputs._fields_:
            setattr(o, name, _ptr(out.get(name)))
        o.status = self._status.data_ptr()
        p = self._params(layer, band, sample_layer, sample_band, sun, chains)
        stream = torch.cuda.current_stream().cuda_stream
        check(self.lib.sky_cuda_adjoint_forward(self.gs.handle, ctypes.byref(self._c_config), ctypes.byref(p),
                                                ctypes.byref(o), ctypes.c_void_p(stream)), self.lib)
        if check_status:
            self._check_status()
        return out

    def backward(self, layer, band, dloss_dfilm, *, sun=None, check_status: bool = True, decorrelate: bool = False,
                 layer_grad: bool = True, chains=None):
        """(dLoss/dlayer_params or None, dLoss/dband_params or None) as float64
        tensors.  decorrelate=True replays chains of another seed than the
        forward's; layer_grad=False skips the layer gradient (band only).
        chains: the buffer a forward at the same parameters and sun filled;
        the replay then skips its first trace of each chain."""
        import torch
        d = dloss_dfilm.reshape(-1).to(torch.float32).contiguous()
        if d.numel() != self.pixels * self.bands:
            raise ValueError("dloss_dfilm must hold pixels * bands values")
        if not layer_grad and band is None:
            raise ValueError("nothing to differentiate: layer_grad=False and no band parameters")
        lg = torch.zeros(self.param_count, dtype=torch.float64, device="cuda") if layer_grad else None
        bg = torch.zeros(self.bands * BAND_PARAMS, dtype=torch.float64, device="cuda") if band is not None else None
        g = SkyAdjointGrads()
        g.dloss_dfilm = d.data_ptr()
        g.layer_grad = _ptr(lg)
        g.band_grad = _ptr(bg)
        g.status = self._status.data_ptr()
        if decorrelate and chains is not None:
            raise ValueError("a decorrelated backward traces other chains than the forward's: no chain buffer")
        stream = torch.cuda.current_stream().cuda_stream
        c = self._c_config
        if decorrelate:
            c = self.config.to_c()
            c.seed = self.config.seed ^ DECORRELATE_SEED
            # the radiance of the backward's own chains from the (lighter) forward kernel,
            # so that the replay traces each chain once and skips those that collected nothing
            chains = self._decorrelated_chains(layer, band, sun, c)
        p = self._params(layer, band, None, None, sun, chains)
        check(self.lib.sky_cuda_adjoint_backward(self.gs.handle, ctypes.byref(c), ctypes.byref(p),
                                                 ctypes.byref(g), ctypes.c_void_p(stream)), self.lib)
        if check_status:
            self._check_status()
        return lg, bg

    def _decorrelated_chains(self, layer, band, sun, c):
        """Chain radiance of config `c` (the decorrelated seed) at these
        parameters, in a buffer the renderer keeps for its next backward."""
        import torch
        if getattr(self, "_dchains", None) is None:
            self._dchains = self.new_chain_buffer()
            self._dsums = torch.empty(self.pixels * self.bands, dtype=torch.float64, device="cuda")
        o = SkyDeviceOutputs()
        o.cell_sum = self._dsums.data_ptr()
        o.status = self._status.data_ptr()
        p = self._params(layer, band, None, None, sun, self._dchains)
        stream = torch.cuda.current_stream().cuda_stream
        check(self.lib.sky_cuda_adjoint_forward(self.gs.handle, ctypes.byref(c), ctypes.byref(p), ctypes.byref(o),
                                                ctypes.c_void_p(stream)), self.lib)
        return self._dchains

    def _jobs(self, suns, config, dlosses=None, chains=None, outputs=None):
        """SkyAdjointJob rows of the renders at `suns` (one each)."""
        n = len(suns)
        jobs = (SkyAdjointJob * n)()
        c = config
        for i, sun in enumerate(suns):
            j = jobs[i]
            j.config = c
            j.sun_direction = (ctypes.c_float * 3)(*(sun if sun is not None else (0.0, 0.0, 0.0)))
            if outputs is not None:
                o = outputs[i]
                for name, _ in SkyDeviceOutputs._fields_:
                    setattr(j.outputs, name, _ptr(o.get(name)))
                j.outputs.status = self._status.data_ptr()
            if dlosses is not None:
                j.dloss_dfilm = dlosses[i].data_ptr()
            if chains is not None and chains[i] is not None:
                ch = chains[i]
                if not (ch.is_cuda and ch.is_contiguous()) or ch.numel() != self.chain_count or \
                        str(ch.dtype) != "torch.float32":
                    raise ValueError(f"chains must be contiguous float32 CUDA tensors of {self.chain_count} values")
                j.chain_radiance = ch.data_ptr()
                j.chain_radiance_len = ch.numel()
        return jobs

    def forward_batch(self, layer, band, suns, *, chains=None, check_status: bool = True, config=None) -> list:
        """One launch (per 32 renders) of the forward at every sun of `suns`
        (unit vectors, None = the scene's): a list of films and cell sums as
        forward() returns them.  chains: a chain-radiance buffer per sun, or
        None."""
        import torch
        cells = self.pixels * self.bands
        outs = [{"cell_sum": torch.empty(cells, dtype=torch.float64, device="cuda"),
                 "cell_sumsq": torch.empty(cells, dtype=torch.float64, device="cuda"),
                 "film": torch.empty(cells, dtype=torch.float32, device="cuda")} for _ in suns]
        jobs = self._jobs(suns, config or self._c_config, chains=chains, outputs=outs)
        p = self._params(layer, band)
        stream = torch.cuda.current_stream().cuda_stream
        check(self.lib.sky_cuda_adjoint_forward_batch(self.gs.handle, jobs, len(suns), ctypes.byref(p),
                                                      ctypes.c_void_p(stream)), self.lib)
        if check_status:
            self._check_status()
        return outs

    def backward_batch(self, layer, band, dlosses, suns, *, check_status: bool = True, decorrelate: bool = False,
                       layer_grad: bool = True, chains=None):
        """Gradient of sum_i Loss_i over the renders at `suns` given each
        dLoss_i/dfilm_i, in one launch per direction (per 32 renders).  With
        decorrelate=True each render's chains come from another seed: their
        radiance is rendered first by the forward kernel (one launch), then
        replayed once."""
        import torch
        if decorrelate and chains is not None:
            raise ValueError("a decorrelated backward traces other chains than the forward's: no chain buffer")
        if not layer_grad and band is None:
            raise ValueError("nothing to differentiate: layer_grad=False and no band parameters")
        ds = [d.reshape(-1).to(torch.float32).contiguous() for d in dlosses]
        for d in ds:
            if d.numel() != self.pixels * self.bands:
                raise ValueError("each dloss_dfilm must hold pixels * bands values")
        lg = torch.zeros(self.param_count, dtype=torch.float64, device="cuda") if layer_grad else None
        bg = torch.zeros(self.bands * BAND_PARAMS, dtype=torch.float64, device="cuda") if band is not None else None
        c = self._c_config
        stream = torch.cuda.current_stream().cuda_stream
        if decorrelate:
            c = self.config.to_c()
            c.seed = self.config.seed ^ DECORRELATE_SEED
            chains = self._decorrelated_chain_batch(layer, band, suns, c)
        jobs = self._jobs(suns, c, dlosses=ds, chains=chains)
        g = SkyAdjointGrads()
        g.layer_grad = _ptr(lg)
        g.band_grad = _ptr(bg)
        g.status = self._status.data_ptr()
        p = self._params(layer, band)
        check(self.lib.sky_cuda_adjoint_backward_batch(self.gs.handle, jobs, len(suns), ctypes.byref(p),
                                                       ctypes.byref(g), ctypes.c_void_p(stream)), self.lib)
        if check_status:
            self._check_status()
        return lg, bg

    def _decorrelated_chain_batch(self, layer, band, suns, c):
        """Chain radiance of config `c` at every sun, from one forward launch,
        in buffers the renderer keeps for its next backward."""
        n = len(suns)
        if len(getattr(self, "_dchain_batch", [])) < n:
            self._dchain_batch = [self.new_chain_buffer() for _ in range(n)]
        chains = self._dchain_batch[:n]
        self.forward_batch(layer, band, suns, chains=chains, check_status=False, config=c)
        return chains

    def bake_majorants(self, layer, band=None):
        """Majorant grid [B, L] of the parameterised medium (device bake)."""
        import torch
        out = torch.empty((self.bands, self.layers), dtype=torch.float32, device="cuda")
        p = self._params(layer, band)
        stream = torch.cuda.current_stream().cuda_stream
        check(self.lib.sky_cuda_bake_majorants(self.gs.handle, ctypes.byref(p), ctypes.c_void_p(out.data_ptr()),
                                               ctypes.c_void_p(stream)), self.lib)
        return out


def _autograd_function():
    import torch

    class SkyRenderFunction(torch.autograd.Function):
        """film = render(layer_params, band_params); backward runs the adjoint kernel."""

        @staticmethod
        def forward(ctx, layer, band, renderer, sun, decorrelate):
            layer_c = layer.detach().contiguous()
            band_c = band.detach().contiguous() if band is not None else None
            # each chain's radiance, so that the backward replays each chain once
            ctx.chains = None if decorrelate else renderer.new_chain_buffer()
            out = renderer.forward(layer_c, band_c, sun=sun, check_status=renderer.check_each_call,
                                   chains=ctx.chains)
            ctx.renderer = renderer
            ctx.sun = sun
            ctx.decorrelate = decorrelate
            ctx.has_band = band is not None
            ctx.save_for_backward(layer_c, band_c if band_c is not None else layer_c)
            cfg = renderer.config
            return out["film"].reshape(cfg.rows, cfg.width, renderer.bands)

        @staticmethod
        def backward(ctx, grad_film):
            layer_c, band_c = ctx.saved_tensors
            band_c = band_c if ctx.has_band else None
            want_layer = ctx.needs_input_grad[0] or band_c is None
            lg, bg = ctx.renderer.backward(layer_c, band_c, grad_film.contiguous(), sun=ctx.sun,
                                           decorrelate=ctx.decorrelate, layer_grad=want_layer,
                                           check_status=ctx.renderer.check_each_call, chains=ctx.chains)
            ctx.chains = None
            gl = lg.to(layer_c.dtype).reshape(layer_c.shape) if lg is not None else None
            gb = bg.to(band_c.dtype).reshape(band_c.shape) if bg is not None else None
            return gl, gb, None, None, None

    return SkyRenderFunction


_FUNCTION = None
_BATCH_FUNCTION = None


def _batch_autograd_function():
    import torch

    class SkyBatchRenderFunction(torch.autograd.Function):
        """films[i] = render(layer_params, band_params, sun_i) for every sun in
        one launch; the backward runs one adjoint launch for all of them."""

        @staticmethod
        def forward(ctx, layer, band, renderer, suns, decorrelate):
            layer_c = layer.detach().contiguous()
            band_c = band.detach().contiguous() if band is not None else None
            ctx.chains = None if decorrelate else [renderer.new_chain_buffer() for _ in suns]
            outs = renderer.forward_batch(layer_c, band_c, suns, chains=ctx.chains,
                                          check_status=renderer.check_each_call)
            ctx.renderer = renderer
            ctx.suns = suns
            ctx.decorrelate = decorrelate
            ctx.has_band = band is not None
            ctx.save_for_backward(layer_c, band_c if band_c is not None else layer_c)
            cfg = renderer.config
            return torch.stack([o["film"].reshape(cfg.rows, cfg.width, renderer.bands) for o in outs])

        @staticmethod
        def backward(ctx, grad_films):
            layer_c, band_c = ctx.saved_tensors
            band_c = band_c if ctx.has_band else None
            want_layer = ctx.needs_input_grad[0] or band_c is None
            grads = [grad_films[i].contiguous() for i in range(grad_films.shape[0])]
            lg, bg = ctx.renderer.backward_batch(layer_c, band_c, grads, ctx.suns, decorrelate=ctx.decorrelate,
                                                 layer_grad=want_layer, check_status=ctx.renderer.check_each_call,
                                                 chains=ctx.chains)
            ctx.chains = None
            gl = lg.to(layer_c.dtype).reshape(layer_c.shape) if lg is not None else None
            gb = bg.to(band_c.dtype).reshape(band_c.shape) if bg is not None else None
            return gl, gb, None, None, None

    return SkyBatchRenderFunction


def render_films(renderer: AdjointRenderer, layer, band=None, suns=(None,), decorrelate: bool = False):
    """Differentiable films [len(suns), H, W, B] (float32) of the renderer's
    config at every sun: one forward launch and, on backward, one adjoint
    launch for all of them (per 32 suns)."""
    global _BATCH_FUNCTION
    if _BATCH_FUNCTION is None:
        _BATCH_FUNCTION = _batch_autograd_function()
    return _BATCH_FUNCTION.apply(layer, band, renderer, list(suns), decorrelate)


def render_film(renderer: AdjointRenderer, layer, band=None, sun=None, decorrelate: bool = False):
    """Differentiable film [H, W, B] (float32) of the renderer's config.

    With decorrelate=True the backward pass traces its own samples (another
    seed) instead of replaying the forward's: the gradient of a loss that is
    nonlinear in the film (e.g. L2) is then free of the correlation between
    the film's noise and its derivative's noise."""
    global _FUNCTION
    if _FUNCTION is None:
        _FUNCTION = _autograd_function()
    return _FUNCTION.apply(layer, band, renderer, sun, decorrelate)


def film_to_xyz(film, scene: Scene):
    """CIE XYZ [H, W, 3] (float64) of a film, with the scene's band weights
    (spectrum_to_xyz_with_weights, spectrum.rs:232-241)."""
    import torch
    w = torch.as_tensor(np.asarray(scene.band_xyz, dtype=np.float64), device=film.device)
    return film.to(torch.float64) @ w
