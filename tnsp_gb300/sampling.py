"""Drop-in mirrors of tetragono's ``SweepSampling``, ``Configuration`` and ``Observer``.

The reference runs one Markov chain per process and calls, once per sample
(tetragono/tetragono/sampling_lattice/gradient.py:331-358)::

    with seed_differ, observer:
        sampling = SweepSampling(state, cut, restrict, hopping)
        sampling.configuration.import_configuration(configs)
        for step in range(total):
            possibility, configuration = sampling()
            observer(possibility, configuration)

The same loop runs unchanged here.  ``SweepSampling`` owns ``chains`` Markov chains on the GPU;
its first call sweeps all of them in one launch (observing every new configuration in the same
kernel when an ``Observer`` is entered on the lattice) and the following calls hand out the other
chains' samples without device work.  ``Observer.__call__`` therefore only checks the pairing: the
accumulation already happened on the device, and ``energy`` / ``gradient`` read the reduced
accumulators.

Only the features of the sweep / E_loc / gradient / natural-gradient path are mirrored.  Restricted
subspaces and custom hopping Hamiltonians are accepted when the restriction depends on the replaced
sites only (as tetraku's ``restrict_Sz`` does): it is evaluated here for every table entry and the
device skips the disallowed ones.  Observer sets take diagonal and off-diagonal operators at any
distance (the replaced configurations' amplitudes come from the device amplitude entry).  No cached
deltas (``NotImplementedError`` where the reference would accept them).
"""
import numpy as np

from .engine import Sampler, estimators, gradient_from
from ._lib import PRECISIONS


def _process_group():
    """(rank, world size, torch.distributed module) of the default process group, or (0, 1, None)."""
    try:
        import torch.distributed as dist
    except ImportError:
        return 0, 1, None
    if not (dist.is_available() and dist.is_initialized()):
        return 0, 1, None
    return dist.get_rank(), dist.get_world_size(), dist


def allreduce_sum(arrays):
    """Sums float64 host arrays over the ranks of the default ``torch.distributed`` group, as the
    reference's ``Observer.__exit__`` sums its accumulators with MPI Allreduce
    (tetragono/tetragono/sampling_lattice/observer.py:89-126).  One collective for all arrays; the
    identity without a group or with one rank."""
    rank, world, dist = _process_group()
    arrays = [np.asarray(a, dtype=np.float64) for a in arrays]
    if world == 1:
        return arrays
    import torch
    flat = torch.from_numpy(np.concatenate([a.ravel() for a in arrays]))
    if dist.get_backend() == "nccl":
        flat = flat.cuda()
    dist.all_reduce(flat, op=dist.ReduceOp.SUM)
    flat = flat.cpu().numpy()
    out, o = [], 0
    for a in arrays:
        out.append(flat[o:o + a.size].reshape(a.shape))
        o += a.size
    return out


def _edge_point(charges, p):
    """The reference's EdgePoint (symmetry, index within its segment) of physical index p, from the
    per-index charges of the physical edge (one segment per charge, in edge order)."""
    q = charges[p]
    return (q, p - charges.index(q))


class _RestrictionView:
    """What a restriction callable reads: ``configuration[l1, l2, orbit]`` as an EdgePoint and
    ``configuration.owner``."""

    def __init__(self, owner, conf, charges):
        self.owner = owner
        self._conf = conf
        self._charges = charges

    def __getitem__(self, key):
        l1, l2, _ = key
        return _edge_point(self._charges, int(self._conf[l1, l2]))


def restriction_flags(owner, tables, restrict, conf):
    """One 0/1 flag per entry of ``tables`` (layout of ``lattice.table_arrays``): whether
    ``restrict(configuration, replacement)`` allows replacing the term's sites, from the entry's input
    values, by its output values (sampling.py:133-136, observer.py:364-367).  It is evaluated on two
    backgrounds (``conf`` and its complement at the other sites); a restriction whose answer depends on
    sites outside the replaced ones raises NotImplementedError (the device cannot call it per proposal)."""
    charges = list(owner.charges[1]) if owner.charges is not None else [0] * owner.P
    conf = np.array(conf, dtype=np.int64).reshape(owner.L1, owner.L2)
    backgrounds = [conf, (owner.P - 1) - conf]
    flags = []
    for positions, table in tables.items():
        for s0 in range(owner.P):
            for s1 in range(owner.P):
                for s_out, _ in table.get((s0, s1), []):
                    replacement = {tuple(p): _edge_point(charges, int(v)) for p, v in zip(positions, s_out)}
                    answers = set()
                    for bg in backgrounds:
                        c = bg.copy()
                        for p, v in zip(positions, (s0, s1)):
                            c[p[0], p[1]] = v
                        answers.add(bool(restrict(_RestrictionView(owner, c, charges), replacement)))
                    if len(answers) != 1:
                        raise NotImplementedError("restrict_subspace depends on sites outside the replaced ones")
                    flags.append(1 if answers.pop() else 0)
    return np.array(flags, dtype=np.uint8)


def default_seeds(chains, seed_base=0):
    """Chain b of rank r gets seed ``seed_base + r * chains + b``: distinct chains on every rank, as the
    reference's SeedDiffer gives every MPI rank its own seed (tetragono/tetragono/utility.py:139-168)."""
    rank, _, _ = _process_group()
    return np.arange(chains, dtype=np.uint64) + np.uint64(seed_base + rank * chains)


class Configuration:
    """One chain's configuration (``Configuration``, tetragono/tetragono/sampling_lattice/lattice.py:27-416),
    as seen by the driver: indexing and export/import of the int64 [L1, L2, orbit] array."""

    def __init__(self, owner, config):
        self.owner = owner
        self._config = np.array(config, dtype=np.int64).reshape(owner.L1, owner.L2)

    def __getitem__(self, l1l2o):
        l1, l2, orbit = l1l2o
        if orbit != 0:
            raise KeyError(l1l2o)
        return int(self._config[l1, l2])

    def export_configuration(self):
        return self._config[:, :, None].copy()

    def valid(self):
        return True


class _PendingImport(Configuration):
    """``SweepSampling.configuration`` before the first sweep: importing sets every chain."""

    def __init__(self, sampling):
        super().__init__(sampling.owner, np.zeros((sampling.owner.L1, sampling.owner.L2), dtype=np.int64))
        self._sampling = sampling

    def import_configuration(self, config):
        config = np.asarray(config, dtype=np.int64)
        if config.ndim == 3:
            config = config[:, :, 0]
        if config.shape != (self.owner.L1, self.owner.L2):
            raise ValueError("configuration shape mismatch")
        self._config = config.copy()
        self._sampling._set_start(config)


class SweepSampling:
    """``SweepSampling(owner, cut_dimension, restrict_subspace, hopping_hamiltonians)``
    (tetragono/tetragono/sampling_lattice/sampling.py:74-193) over ``chains`` GPU chains.

    ``seeds`` (one per chain) seed each chain's mt19937_64 as ``TAT.random.seed`` would; by default
    chain b uses seed ``seed_base + b`` (plus ``rank * chains`` under torch.distributed).  ``discard`` skips that many uniform_real draws first (the
    driver's ``SeedDiffer`` discards one)."""

    def __init__(self, owner, cut_dimension, restrict_subspace=None, hopping_hamiltonians=None, *, chains=1,
                 seeds=None, seed_base=0, discard=0, precision="fp64", device=0):
        self._restrict = restrict_subspace
        self._hopping = hopping_hamiltonians
        self.owner = owner
        self._cut_dimension = cut_dimension
        self.chains = chains
        self.seeds = np.asarray(seeds if seeds is not None else default_seeds(chains, seed_base), dtype=np.uint64)
        if self.seeds.shape != (chains,):
            raise ValueError("one seed per chain")
        self.discard = discard
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self.precision = PRECISIONS[precision]
        self._engine = Sampler(owner, cut_dimension, device=device)
        owner._gpu_engine = self._engine
        self._started = False
        self._buffer = []
        self.configuration = _PendingImport(self)

    def _set_start(self, config):
        if self._restrict is not None or self._hopping is not None:
            tables = self._hopping if self._hopping is not None else self.owner._hamiltonians
            allowed = None
            if self._restrict is not None:
                allowed = restriction_flags(self.owner, tables, self._restrict, config)
            self._engine.set_hopping(self._hopping, allowed)
        self._engine.init_chains(np.asarray(config, dtype=np.int32), self.seeds, discard=self.discard,
                                 precision=self.precision)
        self._start_config = np.array(config)
        self._started = True

    def refresh_all(self):
        """The lattice tensors changed: upload them (chains keep their configurations)."""
        self._engine.upload()

    def __call__(self):
        if not self._started:
            raise RuntimeError("Configuration not initialized")
        if not self._buffer:
            observer = getattr(self.owner, "_active_observer", None)
            observing = observer is not None
            if observing and observer._engine is not self._engine:
                observer._bind(self._engine, self._start_config)
            if self._engine._uploaded_version != self.owner.version:
                self._engine.upload()
            self._engine.sweep(1, observe=observing)
            conf, logp = self._engine.read_chains()
            if observing and (observer._enable_natural or observer._observer_set):
                eloc, _, reweight = self._engine.read_samples(1)
                if observer._enable_natural:
                    observer._samples_e.extend(eloc[0].tolist())
                    observer._samples_w.extend(reweight[0].tolist())
                if observer._observer_set:
                    observer._observe_set(conf, reweight[0])
            self._buffer = [(float(np.exp(lp)), Configuration(self.owner, c), observing) for c, lp in zip(conf, logp)]
            self._buffer.reverse()
        possibility, configuration, observed = self._buffer.pop()
        configuration._observed = observed
        self.configuration = configuration
        return possibility, configuration


class Observer:
    """``Observer`` (tetragono/tetragono/sampling_lattice/observer.py:28-920) for energy and gradient."""

    def __init__(self, owner, *, observer_set=None, enable_energy=False, enable_gradient=False,
                 enable_natural_gradient=False, cache_natural_delta=None, cache_configuration=False,
                 restrict_subspace=None, classical_energy=None):
        # cache_configuration (True or "drop") selects the reference's ConfigurationPool for replaced
        # amplitudes; here they always come from the amplitude entry, so it changes nothing
        if cache_natural_delta or classical_energy is not None:
            raise NotImplementedError("cached natural-gradient deltas and classical energies are not supported")
        self.owner = owner
        self._restrict = restrict_subspace
        # observer_set: {name: {positions: element table}}, tables as the lattice's Hamiltonian tables
        # ({input tuple: [(output tuple, value)]}).  Diagonal elements need the sampled configuration
        # alone; off-diagonal ones need the amplitude of the replaced configuration at any distance,
        # which the reference takes from its ConfigurationPool (lattice.py:473-696) and this observer from
        # the device amplitude entry (tnsp_amplitude) for all samples of a sweep at once
        self._observer_set = {}
        self._has_offdiag = False
        for name, terms in (observer_set or {}).items():
            if name == "energy":
                raise ValueError("the name 'energy' is reserved for the Hamiltonian")
            entries = []
            for positions, table in terms.items():
                positions = tuple(tuple(p) for p in positions)
                if any(p[2] != 0 for p in positions):
                    raise NotImplementedError("only orbit 0 is supported")
                diag, off = {}, {}
                for s_in, outs in table.items():
                    for s_out, value in outs:
                        if tuple(s_out) == tuple(s_in):
                            diag[tuple(s_in)] = diag.get(tuple(s_in), 0.0) + float(value)
                        else:
                            off.setdefault(tuple(s_in), []).append((tuple(s_out), float(value)))
                self._has_offdiag |= bool(off)
                entries.append((positions, diag, off))
            self._observer_set[name] = entries
        if self._has_offdiag and getattr(owner, "fermion", None) is not None:
            raise NotImplementedError("off-diagonal observer sets on fermionic lattices")
        self._set_acc = None
        self._enable_natural = bool(enable_natural_gradient)
        self._enable_energy = enable_energy or enable_gradient or self._enable_natural
        self._enable_gradient = enable_gradient or self._enable_natural
        self._samples_e = []
        self._samples_w = []
        self._engine = None
        self._count = 0
        self._scalars = None
        self._delta = None
        self._edelta = None

    def __enter__(self):
        """``Observer.__enter__``: the accumulators start empty; they are bound to the sampler whose
        first sweep happens inside this context (the driver creates the SweepSampling after entering)."""
        self._engine = None
        self._count = 0
        self._scalars = None
        self._samples_e = []
        self._samples_w = []
        self._set_acc = {name: (np.zeros((len(entries), 3)), np.zeros(3)) for name, entries in self._observer_set.items()}
        self.owner._active_observer = self
        return self

    def _allowed(self, conf, positions, s_out):
        """restrict_subspace(configuration, replacement) of the observer (observer.py:364-367)."""
        if self._restrict is None:
            return True
        charges = getattr(self.owner, "charges", None)
        ch = list(charges[1]) if charges is not None else [0] * self.owner.P
        replacement = {p: _edge_point(ch, int(v)) for p, v in zip(positions, s_out)}
        return bool(self._restrict(_RestrictionView(self.owner, conf, ch), replacement))

    def _offdiag_values(self, confs, keep):
        """Per kept sample i and term (name, k): sum over s' != s of <s'|O|s> psi(s') / psi(s)
        (observer.py:355-389), with psi of the sample and of every replaced configuration from the
        amplitude kernel; terms the observer's restriction forbids (observer.py:364-367) and replaced
        configurations of zero amplitude contribute nothing."""
        requests, replaced = [], []
        for i, b in enumerate(keep):
            conf = confs[b]
            for name, entries in self._observer_set.items():
                for k, (positions, _, off) in enumerate(entries):
                    outs = off.get(tuple(int(conf[p[0], p[1]]) for p in positions))
                    if not outs:
                        continue
                    for s_out, value in outs:
                        if not self._allowed(conf, positions, s_out):
                            continue
                        c = conf.copy()
                        for p, v in zip(positions, s_out):
                            c[p[0], p[1]] = v
                        requests.append((i, name, k, value))
                        replaced.append(c)
        values = {}
        if not replaced:
            return values
        m0, e0 = self._engine.amplitude(confs[keep])
        m1, e1 = self._engine.amplitude(np.array(replaced))
        for (i, name, k, value), mm, ee in zip(requests, m1, e1):
            if m0[i] == 0.0 or mm == 0.0:
                continue
            values[(i, name, k)] = values.get((i, name, k), 0.0) + value * float(np.ldexp(mm / m0[i], int(ee - e0[i])))
        return values

    def _observe_set(self, confs, reweights):
        """Observer.__call__ (observer.py:344-402) for the observer set: per sample with nonzero weight w
        and per term the value x = sum over s' of <s'|O|s> psi(s') / psi(s), summing x w, x w^2 and
        x^2 w^2, and the same for the sum over a name's terms."""
        confs = np.asarray(confs).reshape(-1, self.owner.L1, self.owner.L2)
        keep = [b for b in range(len(confs)) if reweights[b] != 0.0]
        off = self._offdiag_values(confs, keep) if (self._has_offdiag and keep) else {}
        for i, b in enumerate(keep):
            conf, w = confs[b], reweights[b]
            for name, entries in self._observer_set.items():
                acc, whole = self._set_acc[name]
                total = 0.0
                for k, (positions, diag, _) in enumerate(entries):
                    s_in = tuple(int(conf[p[0], p[1]]) for p in positions)
                    x = diag.get(s_in, 0.0)
                    if x != 0.0 and not self._allowed(conf, positions, s_in):
                        x = 0.0  # the reference asks the restriction about the unchanged sites as well
                    x += off.get((i, name, k), 0.0)
                    acc[k] += (x * w, x * w * w, x * x * w * w)
                    total += x
                whole += (total * w, total * w * w, total * total * w * w)

    def restrict_subspace(self, restrict_subspace):
        """``Observer.restrict_subspace`` (observer.py:224-233): E_loc terms that leave the subspace are
        skipped."""
        self._restrict = restrict_subspace

    def _bind(self, engine, start=None):
        if self._engine is not None:
            raise RuntimeError("one observer context observes one SweepSampling")
        self._engine = engine
        if self._restrict is not None:
            engine.restrict_energy(restriction_flags(self.owner, self.owner._hamiltonians, self._restrict, start))
        elif getattr(engine, "energy_restricted", False):
            engine.restrict_energy(None)  # an earlier observer's restriction does not carry over
        engine.keep_holes(self._enable_natural)
        engine.reset_observer()

    def __exit__(self, exc_type, exc_val, exc_tb):
        self.owner._active_observer = None
        if exc_type is not None:
            return False
        if self._engine is not None:
            self._scalars, self._delta, self._edelta = self._reduced(
                *self._engine.read_observer(with_gradient=self._enable_gradient))
        if self._set_acc:
            names = list(self._set_acc)
            flat = np.concatenate([np.concatenate([a.ravel(), w]) for a, w in (self._set_acc[n] for n in names)])
            (flat,) = allreduce_sum([flat])
            pos = 0
            for n in names:
                a, w = self._set_acc[n]
                a[...] = flat[pos:pos + a.size].reshape(a.shape)
                pos += a.size
                w[...] = flat[pos:pos + 3]
                pos += 3
        return False

    def _expect(self, sums):
        """``_expect_and_deviation`` (observer.py:433-469) with the totals of the weights."""
        s = self._read()
        R, RR = s[1], s[2]
        ER, ERR, EERR = sums
        if ER == 0.0 or R == 0.0:
            return 0.0, 0.0
        expect = ER / R
        variance = (EERR - 2 * ERR * expect + RR * expect**2) / R**2
        return expect, (variance**0.5 if variance >= 0.0 else 0.0)

    @property
    def result(self):
        """``Observer.result``: {name: {positions: (expect, deviation)}} of the observer set."""
        return {name: {entry[0]: self._expect(self._set_acc[name][0][k]) for k, entry in enumerate(entries)}
                for name, entries in self._observer_set.items()}

    @property
    def whole_result(self):
        """``Observer.whole_result``: {name: (expect, deviation)} of each name's summed terms, and the
        energy."""
        out = {name: self._expect(self._set_acc[name][1]) for name in self._observer_set}
        if self._enable_energy:
            out["energy"] = self.total_energy
        return out

    def _reduced(self, scalars, delta, edelta):
        """Sum over the ranks of a process group (one collective), as ``Observer.__exit__`` does."""
        if delta is None:
            scalars, = allreduce_sum([scalars])
            return scalars, None, None
        return tuple(allreduce_sum([scalars, delta, edelta]))

    def __call__(self, possibility, configuration):
        if not getattr(configuration, "_observed", False):
            raise RuntimeError("the configuration was sampled outside this observer's context")
        self._count += 1

    def _read(self):
        if self._scalars is None:
            self._scalars, self._delta, self._edelta = self._reduced(
                *self._engine.read_observer(with_gradient=self._enable_gradient))
        return self._scalars

    @property
    def total_energy(self):
        e, d = estimators(self._read(), 1)
        return e, d

    @property
    def energy(self):
        return estimators(self._read(), self.owner.site_number)

    @property
    def gradient(self):
        """2 conj(<E Delta> - <E><Delta>) per site tensor, dense (P, U, D, L, R) arrays."""
        if not self._enable_gradient:
            raise RuntimeError("gradient not enabled")
        scal = self._read()
        return self.owner.unflatten(self._fold(gradient_from(scal, self._delta, self._edelta)))

    def _fold(self, flat):
        """A fermionic lattice's gradient takes its static per-element sign (tnsp_gb300.fermion)."""
        fermion = getattr(self.owner, "fermion", None)
        return flat if fermion is None else fermion.fold_flat(flat)

    def natural_gradient_by_conjugate_gradient(self, step, error):
        """``Observer.natural_gradient_by_conjugate_gradient``
        (tetragono/tetragono/sampling_lattice/observer.py:576-675) for real tensors: conjugate gradient
        on D^T D x = D^T E with D_s = (delta_s - <delta>) sqrt(w_s / W), E_s = (E_loc,s - <E>)
        sqrt(w_s / W), stopped after ``step`` steps or when |r|^2 / |b|^2 < error^2; returns 2 x per site
        (dense arrays).  The per-sample hole rows stay on the device: D v and D^T u are products with
        them there (``tnsp_holes_gemv``), the vector updates run here as in the reference; under a
        process group D^T u and |Dp|^2 are summed over the ranks, as the reference's MPI reductions do."""
        if not self._enable_natural:
            raise RuntimeError("natural gradient not enabled")
        scal = self._read()
        W = scal[1]
        energy = scal[4] / W
        delta = np.asarray(self._delta) / W
        w = np.asarray(self._samples_w)
        param = np.sqrt(w / W)
        En = (np.asarray(self._samples_e) - energy) * param
        eng = self._engine

        def D(v):
            return param * (eng.holes_gemv(v) - np.dot(delta, v))

        def DT(u):
            pu = param * u
            r = eng.holes_gemv(pu, transpose=True) - delta * pu.sum()
            (r,) = allreduce_sum([r])
            return r

        b = DT(En)
        b_square = np.dot(b, b)
        x = np.zeros_like(b)
        r = b - DT(D(x))
        p = r
        r_square = np.dot(r, r)
        t = 0
        while True:
            if t == step:
                break
            if error != 0.0 and error**2 > r_square / b_square:
                break
            Dp = D(p)
            (dpdp,) = allreduce_sum([np.array([np.dot(Dp, Dp)])])
            alpha = r_square / dpdp[0]
            x = x + alpha * p
            r = r - alpha * DT(Dp)
            new_r_square = np.dot(r, r)
            beta = new_r_square / r_square
            r_square = new_r_square
            p = r + beta * p
            t += 1
        self.natural_gradient_steps = t
        return self.owner.unflatten(self._fold(2 * x))

    def natural_gradient_by_direct_pseudo_inverse(self, r_pinv, a_pinv, libraries=None):
        """``Observer.natural_gradient_by_direct_pseudo_inverse`` (observer.py:697-907) in one process, the
        equation of its single-process form (observer.py:902-907): with D_s = delta_s - <delta> over the
        kept samples (unweighted rows) and E_s = E_loc,s - <E>, T = D D^T = U diag(L) U^T,
        L^+ = 1 / (L (1 + ((r_pinv max L + a_pinv) / L)^6)) for L > 0 (0 otherwise), and the result
        2 D^T U L^+ U^T E per site.  T is built from the rows kept on the device: H H^T in one product
        (``tnsp_holes_gram``) and the mean correction with H delta (``tnsp_holes_gemv``); the reference distributes the samples with ScaLAPACK, so several ranks
        raise NotImplementedError here (use the conjugate gradient).  ``libraries`` is accepted and not
        used."""
        if not self._enable_natural:
            raise RuntimeError("natural gradient not enabled")
        if _process_group()[1] > 1:
            raise NotImplementedError("the pseudo-inverse natural gradient runs in one process; use the conjugate "
                                      "gradient with several ranks")
        scal = self._read()
        W = scal[1]
        delta = np.asarray(self._delta) / W
        En = np.asarray(self._samples_e) - scal[4] / W
        eng = self._engine
        # T = D D^T with D = H - 1 delta^T: H H^T in one device product, then the mean correction
        u = eng.holes_gemv(delta)                                     # H delta
        T = eng.holes_gram() - u[:, None] - u[None, :] + np.dot(delta, delta)
        T = 0.5 * (T + T.T)
        L, U = np.linalg.eigh(T)
        num = r_pinv * L[-1] + a_pinv
        safe = np.where(L > 0, L, 1.0)
        Linv = np.where(L > 0, 1.0 / (safe * (1.0 + (num / safe)**6)), 0.0)
        y = U @ (Linv * (U.T @ En))
        x = 2 * (eng.holes_gemv(y, transpose=True) - delta * y.sum())
        return self.owner.unflatten(self._fold(x))

    @property
    def instability(self):
        s = self._read()
        N, R, RR = s[0], s[1], s[2]
        expect = R / N
        var = RR / N - expect**2
        return (var**0.5 if var > 0 else 0.0) / expect

    def normalize_lattice(self):
        """``Observer.normalize_lattice`` (observer.py:909-920): rescale every site tensor by
        exp(mean log|ws| / site_number)."""
        s = self._read()
        mean_log_ws = s[3] / s[0]
        param = np.exp(mean_log_ws / self.owner.site_number)
        for l1, l2 in self.owner.sites():
            self.owner[l1, l2] = self.owner[l1, l2] / param
