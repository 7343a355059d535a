"""Learned surrogate of the fused hydrogen-bonding + cross-stacking pair term.

A 7 -> 64 -> 64 -> 64 -> 1 SiLU MLP per pair class (complementary bases, which
hydrogen-bond, and the rest, which only cross-stack) maps the base-base geometry of a
pair (BASE-BASE distance and the cosines c1, c2, c3, c4, c7, c8 of the reference's
base-base evaluator, src/OxDNABaseBase.h:74-121) to its energy. Forces and torques come
from the network's analytic input gradient. BF16 weights on the tensor cores, FP32
accumulation; trained by the library's own kernels on samples the plain evaluator
produces along its own trajectories. The reference has no learned part: this is an
extension, used only while audits by the plain evaluator keep the sampled error of the
term's energy under a tolerance (the plain evaluator stays the fallback and the
yardstick).

Device buffers are torch CUDA tensors (plumbing only); every computation runs in
``liboxdna_gb300.so``.
"""

import ctypes as C

import numpy as np

from . import _abi

N_FEATURES = 7
HIDDEN = 64
P = _abi.MLP_PARAMS
# offsets of one class's FP32 masters (see include/oxdna_gb300.h)
OFF = dict(W1=0, b1=1024, W2=1088, b2=5184, W3=5248, b3=9344, w4=9408, b4=9472)


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def init_params(seed=0):
    """He-style random masters for both classes (2 x P floats)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = np.zeros((2, P), np.float32)
    for c in range(2):
        w1 = np.zeros((64, 16), np.float32)
        w1[:, :N_FEATURES] = rng.normal(0.0, np.sqrt(2.0 / N_FEATURES), (64, N_FEATURES))
        out[c, OFF["W1"]:OFF["W1"] + 1024] = w1.ravel()
        out[c, OFF["W2"]:OFF["W2"] + 4096] = rng.normal(0.0, np.sqrt(2.0 / 64), 4096)
        out[c, OFF["W3"]:OFF["W3"] + 4096] = rng.normal(0.0, np.sqrt(2.0 / 64), 4096)
        out[c, OFF["w4"]:OFF["w4"] + 64] = rng.normal(0.0, np.sqrt(1.0 / 64), 64)
    return out


def unpack(params):
    """Masters of one class (P floats) -> dict of arrays (W1 is 64 x 16)."""
    p = np.asarray(params, np.float64)
    return dict(W1=p[0:1024].reshape(64, 16), b1=p[1024:1088], W2=p[1088:5184].reshape(64, 64),
                b2=p[5184:5248], W3=p[5248:9344].reshape(64, 64), b3=p[9344:9408],
                w4=p[9408:9472], b4=p[9472])


class Network:
    """The surrogate network (both classes) on the GPU."""

    def __init__(self, params=None, seed=0):
        L = _abi.lib()
        h = C.c_void_p()
        _abi.check(L.oxg_mlp_create(C.byref(h)), "oxg_mlp_create")
        self._h = h
        self.norm = [None, None]
        self.set_params(init_params(seed) if params is None else params)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                _abi.lib().oxg_mlp_destroy(self._h)
                self._h = None
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_params(self, params):
        p = np.ascontiguousarray(params, np.float32).reshape(2, P)
        _abi.check(_abi.lib().oxg_mlp_set_params(self._h, p.ctypes.data), "oxg_mlp_set_params")

    def get_params(self):
        p = np.zeros((2, P), np.float32)
        _abi.check(_abi.lib().oxg_mlp_get_params(self._h, p.ctypes.data), "oxg_mlp_get_params")
        return p

    def set_normalization(self, cls, mu, sd, e_scale, e_shift):
        mu = np.ascontiguousarray(mu, np.float32)
        inv = np.ascontiguousarray(1.0 / np.asarray(sd, np.float64), np.float32)
        _abi.check(_abi.lib().oxg_mlp_set_normalization(self._h, int(cls), mu.ctypes.data, inv.ctypes.data,
                                                        float(e_scale), float(e_shift)),
                   "oxg_mlp_set_normalization")
        self.norm[cls] = (mu.astype(np.float64), inv.astype(np.float64), float(e_scale), float(e_shift))

    def fit_normalization(self, feats, energy):
        """Input mean / sd and output scale / shift of each class from a data set
        (torch tensors or arrays: feats n x 8, energy n)."""
        f = _np(feats)
        e = _np(energy)
        for c in (0, 1):
            m = f[:, 7] == c
            if not m.any():
                self.set_normalization(c, np.zeros(7), np.ones(7), 1.0, 0.0)
                continue
            x = f[m, :7].astype(np.float64)
            sd = x.std(axis=0)
            sd[sd < 1e-6] = 1.0
            es = float(e[m].std()) or 1.0
            self.set_normalization(c, x.mean(axis=0), sd, es, float(e[m].mean()))

    def calibrate(self, feats, energy):
        """Shift each class's output so that its mean pair-energy error over a data set
        (the pair distribution the network will meet in MD) is zero: a systematic error
        of the pair energies adds up over every pair of the term, random errors largely
        cancel. Returns the per-class shifts applied."""
        import torch
        shifts = []
        for c in (0, 1):
            m = feats[:, 7] == c
            if int(m.sum()) == 0 or self.norm[c] is None:
                shifts.append(0.0)
                continue
            resid = (self.energies(feats[m].contiguous()) - energy[m]).to(torch.float64)
            d = float(resid.mean())
            mu, inv, es, sh = self.norm[c]
            self.set_normalization(c, mu, 1.0 / inv, es, sh - d)
            shifts.append(-d)
        return shifts

    def gradient(self, cls, feats, target, idx):
        """Loss gradient (P floats) and sum of squared errors for a minibatch (torch
        tensors on the GPU: feats n x 8 float32, target n float32, idx int32)."""
        g = np.zeros(P, np.float32)
        sse = C.c_double()
        _abi.check(_abi.lib().oxg_mlp_gradient(self._h, int(cls), _ptr(feats), _ptr(target), _ptr(idx),
                                               int(idx.numel()), g.ctypes.data, C.byref(sse), None),
                   "oxg_mlp_gradient")
        return g, sse.value

    def predict(self, cls, feats):
        """Network output y and dy/dx' (normalised units) of contiguous samples of one
        class (feats: torch n x 8 float32 on the GPU)."""
        import torch
        n = int(feats.shape[0])
        y = torch.empty(n, dtype=torch.float32, device=feats.device)
        d = torch.empty((n, N_FEATURES), dtype=torch.float32, device=feats.device)
        _abi.check(_abi.lib().oxg_mlp_predict(self._h, int(cls), _ptr(feats), n, _ptr(y), _ptr(d), None),
                   "oxg_mlp_predict")
        return y, d

    def energies(self, feats):
        """Surrogate pair energies of a data set (both classes)."""
        import torch
        out = torch.empty(int(feats.shape[0]), dtype=torch.float32, device=feats.device)
        for c in (0, 1):
            m = feats[:, 7] == c
            if int(m.sum()) == 0:
                continue
            y, _ = self.predict(c, feats[m].contiguous())
            _, _, es, sh = self.norm[c]
            out[m] = y * es + sh
        return out

    def train(self, feats, energy, epochs=10, batch=4096, lr=2e-3, lr_end=5e-5, seed=0,
              log=None):
        """Adam on the mean squared energy error (normalised units) of each class, with a
        cosine learning-rate decay; returns the per-epoch mean training loss."""
        import torch
        L = _abi.lib()
        gen = torch.Generator(device=feats.device)
        gen.manual_seed(seed)
        cls_idx = [torch.nonzero(feats[:, 7] == c).flatten().to(torch.int32) for c in (0, 1)]
        steps_per_epoch = sum((int(ci.numel()) + batch - 1) // batch for ci in cls_idx)
        total = max(1, epochs * steps_per_epoch)
        history = []
        step = 0
        sse = C.c_double()
        for ep in range(epochs):
            tot, cnt = 0.0, 0
            for c in (0, 1):
                ci = cls_idx[c]
                n = int(ci.numel())
                if n == 0:
                    continue
                perm = ci[torch.randperm(n, generator=gen, device=feats.device)].contiguous()
                for b0 in range(0, n, batch):
                    nb = min(batch, n - b0)
                    frac = step / total
                    rate = lr_end + 0.5 * (lr - lr_end) * (1.0 + np.cos(np.pi * frac))
                    last = b0 + batch >= n
                    _abi.check(L.oxg_mlp_train_step(self._h, c, _ptr(feats), _ptr(energy),
                                                    C.c_void_p(perm.data_ptr() + 4 * b0), nb,
                                                    float(rate), C.byref(sse) if last else None, None),
                               "oxg_mlp_train_step")
                    step += 1
                    if last:
                        tot += sse.value
                        cnt += nb
            history.append(tot / max(cnt, 1))
            if log:
                log(f"epoch {ep}: loss {history[-1]:.3e}")
        return history

    def save(self, path):
        np.savez(path, params=self.get_params(),
                 norm=np.array([np.concatenate([n[0], n[1], [n[2], n[3]]]) for n in self.norm]))

    @classmethod
    def load(cls, path):
        d = np.load(path)
        net = cls(params=d["params"])
        for c in (0, 1):
            v = d["norm"][c]
            net.set_normalization(c, v[:7], 1.0 / v[7:14], v[14], v[15])
        return net


def _np(t):
    try:
        return t.detach().cpu().numpy()
    except AttributeError:
        return np.asarray(t)


def samples(sim, max_n=200000):
    """(feats n x 8, energy n) torch tensors of every fused HB + CS pair of a runtime
    Simulation's current state that passes the zero-factor tests (the plain
    evaluator's energies)."""
    import torch
    sim._attach()
    feats = torch.empty((max_n, 8), dtype=torch.float32, device="cuda")
    energy = torch.empty(max_n, dtype=torch.float32, device="cuda")
    n = C.c_int()
    _abi.check(_abi.lib().oxg_system_hbx_samples(sim._sys, max_n, _ptr(feats), _ptr(energy), C.byref(n)),
               "oxg_system_hbx_samples")
    return feats[:n.value].clone(), energy[:n.value].clone()


def training_set(n_target=4_000_000, temperatures=(280, 290, 300, 310, 320, 330, 340, 350, 360),
                 n_dup=200, n_bp=20, box=100.0, equil=0, every=200,
                 early=(5, 10, 15, 20, 30, 40, 50, 60, 70, 80, 90),
                 per_snapshot=5000, built_weight=0.08, seed=11, log=None):
    """Pair geometries from trajectories of the 8000-nt duplex system (200 x 20 bp,
    box 100) at each temperature (oxDNA2, fused forces, Langevin dt 0.003): a random
    subset of at most `per_snapshot` of the queued pairs at step `equil` (default 0: the
    built duplexes and their relaxation are part of what an MD run meets), at the steps
    `early` after it (the relaxation from the built geometry, where the pair geometries
    change fastest) and then every `every` steps, until the set holds n_target pairs
    (spread evenly over the temperatures).

    With equil = 0 the first snapshot, the built duplexes, is repeated to make up
    `built_weight` of each temperature's pairs: every base pair of a built duplex sits at
    one geometry, the state every run from built structures starts from and a common
    read-out, where the network's pointwise error adds up over all pairs instead of
    averaging out (at the weight of plain time sampling, ~1%, that error was 1-4e-4 of the
    term's energy; at ~8%, 2e-6 in an emulation of the training on the CPU, with the
    errors on later states unchanged)."""
    import torch

    from . import io, runtime
    from .model import dna1, dna2
    per_t = n_target // len(temperatures)
    fs, es = [], []
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    for k, T in enumerate(temperatures):
        s = io.duplex_system(n_dup, n_bp, box, seed=seed + k)
        forces, _ = dna2.forces(temperature=T, fused=True)
        sim = runtime.Simulation(device=runtime.device.GPU(), seed=seed + 100 + k)
        sim.create_state_from_snapshot(io.system_snapshot(s))
        lang = runtime.md.methods.Langevin(filter=runtime.filter.All(), kT=dna1.kT_from_temperature(T))
        sim.operations.integrator = runtime.md.Integrator(dt=0.003, integrate_rotational_dof=True,
                                                          forces=forces, methods=[lang])
        sim.run(equil)
        got = 0
        t_now = 0
        marks = [t for t in early if 0 < t < every]
        while got < per_t:
            f, e = samples(sim)
            if per_snapshot and f.shape[0] > per_snapshot:
                sel = torch.randperm(int(f.shape[0]), generator=gen, device=f.device)[:per_snapshot]
                f, e = f[sel], e[sel]
            if t_now == 0 and equil == 0 and built_weight > 0:
                reps = max(1, int(round(built_weight * per_t / max(int(f.shape[0]), 1))))
                f, e = f.repeat(reps, 1), e.repeat(reps)
            take = min(int(f.shape[0]), per_t - got)
            fs.append(f[:take])
            es.append(e[:take])
            got += take
            t_next = marks.pop(0) if marks else (t_now // every + 1) * every
            sim.run(t_next - t_now)
            t_now = t_next
        if log:
            log(f"T = {T} K: {got} pairs")
        del sim
    return torch.cat(fs), torch.cat(es)
