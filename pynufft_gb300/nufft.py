"""``NUFFT``: the GB300 drop-in for the reference class ``pynufft.NUFFT``.

Surface follows nufft/__init__.py:496-738 of the reference (pynufft 2025.2.1):
``plan(om, Nd, Kd, Jd[, ft_axes][, batch])`` returns 0, ``forward``,
``adjoint``, ``selfadjoint``, ``solve(y, 'cg', maxiter=...)`` and the stage
methods ``x2xx``, ``xx2k``, ``k2y``, ``y2k``, ``k2xx``, ``xx2x``, ``k2y2k``,
``xx2k_one2one``, ``k2xx_one2one``.  The ``batch`` argument follows the
deprecated device class (linalg/nufft_hsa.py:152-242): x is Nd+(batch,),
k is Kd+(batch,), y is (M, batch), coils share the points.

Every transform runs on the GPU through the C ABI of libpynufft_gb300.so;
there is no CPU path.  Inputs may be numpy arrays (results come back as
numpy complex64), CUDA torch tensors (results stay on the device, no host
synchronisation) or CPU torch tensors (copied in and out; pinned memory makes
both copies asynchronous).  The reference's CPU path returns complex128 from
``forward``/``k2y``/``y2k``; this one returns complex64 everywhere.
"""
from __future__ import annotations

import ctypes
from ctypes import c_int, c_int64, c_void_p

import numpy

from . import _lib
from .plan_params import alpha_fit


def _torch():
    import torch
    return torch


class NUFFT:
    """Min-max NUFFT on one GB300 (see the module docstring)."""

    def __init__(self, device_indx=None, legacy=None):
        torch = _torch()
        if not torch.cuda.is_available():
            raise RuntimeError('pynufft_gb300 needs a CUDA device; it has no CPU fallback')
        if device_indx is None:
            dev = torch.device('cuda', torch.cuda.current_device())
        elif isinstance(device_indx, int):
            dev = torch.device('cuda', device_indx)
        elif isinstance(device_indx, (str, torch.device)):
            dev = torch.device(device_indx)
        else:
            # a device description from the reference's helper.device_list():
            # the operator always runs on the current CUDA device
            dev = torch.device('cuda', torch.cuda.current_device())
        self.device = dev
        self.dtype = numpy.complex64
        self.processor = 'gb300'
        self.debug = 0
        self.Nd = ()
        self.Kd = ()
        self.Jd = ()
        self.ndims = 0
        self.ft_axes = ()
        self.batch = None
        self.ninst = 1
        self._plan = None
        self._points = None
        self._twins = []
        self._lane_streams = []
        self.fft = 'auto'
        self._lib = _lib.load()

    # ------------------------------------------------------------------ plan
    def plan(self, om, Nd, Kd, Jd, ft_axes=None, batch=None, deterministic=False,
             bins=None, max_sub_points=None, autotune=False, fft='auto'):
        """Plan for the points ``om`` (M x ndim radians).

        Argument checks follow helper.plan (src/_helper/helper.py:644-654):
        ``TypeError`` when Nd/Kd/Jd are not tuples, ``KeyError`` when their
        lengths differ.  ``deterministic=True`` selects the bitwise-reproducible
        gridding mode.  ``bins``/``max_sub_points`` override the gridding bin
        shape; ``autotune=True`` applies the cached best setting for this
        geometry and point density, or searches once (``pynufft_gb300.autotune``).
        ``fft`` picks the image <-> spectrum transform: ``'cufft'`` cuFFT
        everywhere; ``'auto'`` (the default) the library's own passes where
        they are faster than cuFFT on a GB300 -- one coil with every Kd 256
        and every Nd 128 or 256, and a multiple of 8 coils (one instance,
        2D/3D) with every Kd in {128, 160, 192, 256, 320, 384, 512, 640}, the
        coil-batched passes on the coil-fastest layout -- and cuFFT
        elsewhere; ``'own'`` as ``'auto'``, plus the own pruned power-of-two
        passes on any one-coil 2D/3D plan whose Kd are powers of two.  Returns 0.
        """
        self._check_shapes(Nd, Kd, Jd)
        if fft not in ('auto', 'cufft', 'own'):
            raise ValueError("fft must be 'auto', 'cufft' or 'own'")
        ndim = len(Nd)
        if ft_axes is not None and tuple(sorted(ft_axes)) != tuple(range(ndim)):
            raise NotImplementedError('pynufft_gb300 transforms over all axes (ft_axes=None)')
        B = 1 if batch is None else int(batch)
        if B < 1:
            raise ValueError('batch must be a positive integer')
        st = self._plan_common([om], Nd, Kd, Jd, batch, B, 1, deterministic, bins,
                               max_sub_points, fft)
        if autotune:
            self._autotune([om])
        return st

    def plan_many(self, om_list, Nd, Kd, Jd, batch=None, deterministic=False, bins=None,
                  max_sub_points=None, autotune=False):
        """Plan ``len(om_list)`` independent instances that share Nd/Kd/Jd but
        have their own points (uneven M).  Every transform then runs all
        instances in the same kernel launches: x is (ninst,)+Nd[+(batch,)],
        k is (ninst,)+Kd[+(batch,)] and y concatenates the instances' samples
        in order.  Returns 0."""
        self._check_shapes(Nd, Kd, Jd)
        if len(om_list) < 1:
            raise ValueError('om_list is empty')
        B = 1 if batch is None else int(batch)
        st = self._plan_common(list(om_list), Nd, Kd, Jd, batch, B, len(om_list),
                               deterministic, bins, max_sub_points)
        if autotune:
            self._autotune(list(om_list))
        return st

    def _autotune(self, oms):
        from . import autotune as at
        choice = at.cached(self)
        if choice is not None:
            at.apply(self, oms, choice)
        else:
            at.tune(self, oms if len(oms) > 1 else oms[0])

    @staticmethod
    def _check_shapes(Nd, Kd, Jd):
        if type(Nd) != tuple:
            raise TypeError('Nd must be tuple, e.g. (256, 256)')
        if type(Kd) != tuple:
            raise TypeError('Kd must be tuple, e.g. (512, 512)')
        if type(Jd) != tuple:
            raise TypeError('Jd must be tuple, e.g. (6, 6)')
        if len(Nd) != len(Kd) or len(Nd) != len(Jd):
            raise KeyError('Nd, Kd, Jd must be in the same length, e.g. '
                           'Nd=(256,256),Kd=(512,512),Jd=(6,6)')

    def _plan_common(self, oms, Nd, Kd, Jd, batch, B, ninst, deterministic, bins, max_sub,
                     fft='auto'):
        torch = _torch()
        ndim = len(Nd)
        flags = _lib.NUFFT_FLAG_DETERMINISTIC if deterministic else 0
        if fft == 'own':
            flags |= _lib.NUFFT_FLAG_OWN_FFT
        elif fft == 'cufft':
            flags |= _lib.NUFFT_FLAG_CUFFT
        key = (tuple(Nd), tuple(Kd), tuple(Jd), B, ninst, flags,
               None if bins is None else tuple(bins), max_sub)
        reuse = (self._plan is not None and getattr(self, '_key', None) == key
                 and getattr(self, '_maps', None) is None)
        with torch.cuda.device(self.device):
            if reuse:
                # same geometry: keep the plan (FFT plans, scaling factors and
                # interpolator coefficients); only the points are replaced
                h = self._plan
            else:
                self.release()
                h = c_void_p()
                _lib.check(self._lib.nufft_plan_create(ndim, _lib.int_array(Nd), _lib.int_array(Kd),
                                                       _lib.int_array(Jd), B, ninst, flags,
                                                       ctypes.byref(h)), 'plan')
                self._plan = h
                self._alpha = []
                for d in range(ndim):
                    a, L = alpha_fit(int(Nd[d]), int(Jd[d]), int(Kd[d]))
                    self._alpha.append((a, L))
                    buf = (ctypes.c_float * 16)(*([float(v) for v in a] + [0.0] * (16 - a.size)))
                    _lib.check(self._lib.nufft_plan_set_alpha(h, d, buf, int(L)), 'plan')
                if bins is not None or max_sub is not None:
                    bs = _lib.int_array(bins) if bins is not None else None
                    _lib.check(self._lib.nufft_plan_set_bins(h, bs, int(max_sub or 0)), 'plan')
                self._key = None
                self._sn_cache = None
            counts = []
            parts = []
            on_dev = False
            for om in oms:
                om_t = self._om_tensor(om, ndim)
                counts.append(om_t.shape[0])
                parts.append(om_t)
            if any(p.is_cuda for p in parts):
                om_all = torch.cat([p.to(self.device) for p in parts]).contiguous()
                on_dev = True
                ptr = om_all.data_ptr()
            else:
                om_all = numpy.ascontiguousarray(numpy.concatenate([p.numpy() for p in parts]))
                ptr = om_all.ctypes.data
            cnt = (c_int64 * ninst)(*counts)
            _lib.check(self._lib.nufft_set_points(h, cnt, c_void_p(ptr), 1 if on_dev else 0,
                                                  self._stream()), 'plan')
            self._key = key
            self._points = (om_all, tuple(counts))   # a copy, for run_many's twin plans
            self._drop_twins()
        self.fft = fft
        self.Nd, self.Kd, self.Jd = tuple(Nd), tuple(Kd), tuple(Jd)
        self.ndims = ndim
        self.ft_axes = tuple(range(ndim))
        self.batch = batch
        self.B = B
        self.ninst = ninst
        self.counts = tuple(int(c) for c in counts)
        self.M = (int(sum(counts)),)
        self.deterministic = bool(deterministic)
        self.Kdprod = int(numpy.prod(Kd))
        self.Jdprod = int(numpy.prod(Jd))
        self.st = {'M': numpy.int32(sum(counts)), 'Nd': self.Nd, 'Kd': self.Kd, 'Jd': self.Jd}
        if getattr(self, '_sn_cache', None) is None:
            self._sn_cache = self._host_sn()
        self.sn = self._sn_cache
        return 0

    def _om_tensor(self, om, ndim):
        torch = _torch()
        if isinstance(om, torch.Tensor):
            t = om.detach().to(torch.float64)
        else:
            t = torch.from_numpy(numpy.ascontiguousarray(numpy.asarray(om, dtype=numpy.float64)))
        if t.dim() == 1 and ndim == 1:
            t = t.reshape(-1, 1)
        if t.dim() != 2 or t.shape[1] != ndim:
            raise ValueError(f'om must be (M, {ndim}), got {tuple(t.shape)}')
        return t.contiguous()

    def _host_sn(self):
        """The Kronecker product of the per-axis scaling factors (Nd, complex64),
        as the reference's ``sn`` attribute (nufft/_nufft_class_methods_cpu.py:84)."""
        sn = numpy.ones(())
        for d in range(self.ndims):
            N, J, K = self.Nd[d], self.Jd[d], self.Kd[d]
            al, Lin = self._alpha[d]
            ain = (ctypes.c_float * 16)(*([float(v) for v in al] + [0.0] * (16 - al.size)))
            a = (ctypes.c_float * 16)()
            L = c_int()
            snd = (ctypes.c_double * N)()
            T = (ctypes.c_double * (J * J))()
            _lib.check(self._lib.nufft_axis_params(N, J, K, ain, int(Lin), a, ctypes.byref(L),
                                                   snd, T), 'sn')
            shp = [1] * self.ndims
            shp[d] = N
            sn = sn * numpy.frombuffer(snd, dtype=numpy.float64).reshape(shp)
        return numpy.asarray(sn.astype(numpy.complex64), order='C')

    def release(self):
        """Free the plan's device memory (nufft/_nufft_class_methods_device.py:653-683)."""
        self._drop_twins()
        if getattr(self, '_plan', None) is not None:
            self._lib.nufft_plan_destroy(self._plan)
            self._plan = None
        self._key = None
        self._maps = None
        self._points = None

    def _drop_twins(self):
        for t in getattr(self, '_twins', None) or ():
            t.release()
        self._twins = []

    def _twin(self):
        """Another operator with this one's points and settings and its own
        device buffers, so that a second stream can transform at the same
        time (run_many's lanes)."""
        torch = _torch()
        om_all, counts = self._points
        Nd, Kd, Jd, B, ninst, flags, bins, max_sub = self._key
        if isinstance(om_all, torch.Tensor):
            oms = list(torch.split(om_all, list(counts)))
        else:
            oms = numpy.split(om_all, numpy.cumsum(counts)[:-1])
        t = NUFFT(self.device)
        t._plan_common(oms, Nd, Kd, Jd, self.batch, B, ninst,
                       bool(flags & _lib.NUFFT_FLAG_DETERMINISTIC), bins, max_sub, self.fft)
        k2y, y2k = getattr(self, 'methods', (None, None))
        if k2y is not None or y2k is not None:
            t.set_methods(k2y, y2k)
        return t

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    K2Y_METHODS = {'zteam': 1, 'point': 2, 'tile': 3, 'tile_point': 4}
    Y2K_METHODS = {'zteam': 1, 'point': 2, 'global': 3}

    def set_methods(self, k2y=None, y2k=None):
        """Choose the lane mapping of the interpolation/gridding kernels for
        plans with fewer than 8 coils: k2y in {'tile', 'tile_point', 'zteam', 'point'},
        y2k in {'zteam', 'point', 'global'}; None keeps the default."""
        km = 0 if k2y is None else self.K2Y_METHODS[k2y]
        ym = 0 if y2k is None else self.Y2K_METHODS[y2k]
        _lib.check(self._lib.nufft_plan_set_methods(self._plan, km, ym), 'set_methods')
        self.methods = (k2y, y2k)
        self._drop_twins()

    def check(self):
        """Synchronise the plan's stream and raise NufftError if a kernel gave up
        a bounded wait for its asynchronous loads since the last check
        (nufft_plan_check)."""
        _lib.check(self._lib.nufft_plan_check(self._plan, self._stream()), 'check')

    def info(self):
        m, ns, by = c_int64(), c_int64(), c_int64()
        _lib.check(self._lib.nufft_plan_info(self._plan, ctypes.byref(m), ctypes.byref(ns),
                                             ctypes.byref(by)), 'info')
        return {'M': m.value, 'subproblems': ns.value, 'device_bytes': by.value}

    # ------------------------------------------------------------- plumbing
    def _stream(self):
        torch = _torch()
        return c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def _shape(self, kind):
        lead = (self.ninst,) if self.ninst > 1 else ()
        tail = (self.batch,) if self.batch is not None else ()
        if kind == 'x':
            return lead + self.Nd + tail
        if kind == 'k':
            return lead + self.Kd + tail
        return self.M + tail

    def _in(self, a, kind):
        """-> (device complex64 tensor, how to return the result)."""
        torch = _torch()
        if self._plan is None:
            raise RuntimeError('plan() has not been called')
        shape = self._shape(kind)
        if isinstance(a, torch.Tensor):
            if tuple(a.shape) != shape:
                raise ValueError(f'expected shape {shape}, got {tuple(a.shape)}')
            if a.is_cuda:
                return a.to(self.device, torch.complex64).contiguous(), ('cuda', None)
            t = a.to(torch.complex64)
            pinned = t.is_pinned()
            d = t.to(self.device, non_blocking=pinned).contiguous()
            return d, ('cpu', pinned)
        arr = numpy.asarray(a)
        if arr.shape != shape:
            raise ValueError(f'expected shape {shape}, got {arr.shape}')
        arr = numpy.ascontiguousarray(arr, dtype=numpy.complex64)
        return torch.from_numpy(arr).to(self.device), ('numpy', None)

    def _out(self, t, how):
        torch = _torch()
        kind, pinned = how
        if kind == 'cuda':
            return t
        if kind == 'cpu':
            if pinned:
                o = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                o.copy_(t, non_blocking=True)
                torch.cuda.current_stream(self.device).synchronize()
                return o
            return t.cpu()
        return t.cpu().numpy()

    def _empty(self, kind):
        torch = _torch()
        return torch.empty(self._shape(kind), dtype=torch.complex64, device=self.device)

    def _mapped(self, t):
        """Device address of a pinned CPU tensor mapped into the device, or None."""
        dev = c_void_p()
        if self._lib.nufft_mapped_pointer(c_void_p(t.data_ptr()), ctypes.byref(dev)) != _lib.NUFFT_OK:
            return None
        return dev

    def _call(self, fn, a, kin, kout, name):
        torch = _torch()
        # pinned CPU images of one-coil plans are read (kin 'x') and written
        # (kout 'x') by the streaming image kernels in place over the host
        # link, without a copy.  (The coil-major image kernels of several
        # coils stride over the coils: through the link that ran 40x slower
        # than a copy, 1.3 ms against 31 us per 32-coil 320^2 crop.)
        host_in = (kin == 'x' and self.B == 1 and isinstance(a, torch.Tensor) and not a.is_cuda
                   and a.is_pinned() and a.dtype == torch.complex64 and a.is_contiguous()
                   and tuple(a.shape) == self._shape('x'))
        inptr = self._mapped(a) if host_in else None
        if inptr is not None:
            how = ('cpu', True)
        else:
            d, how = self._in(a, kin)
            inptr = c_void_p(d.data_ptr())
        out, outptr = None, None
        if kout == 'x' and how == ('cpu', True) and self.B == 1:
            out = torch.empty(self._shape('x'), dtype=torch.complex64, pin_memory=True)
            outptr = self._mapped(out)
        if outptr is None:
            out = self._empty(kout)
            outptr = c_void_p(out.data_ptr())
        with torch.cuda.device(self.device):
            _lib.check(fn(self._plan, inptr, outptr, self._stream()), name)
            if not out.is_cuda:
                torch.cuda.current_stream(self.device).synchronize()
                return out
        return self._out(out, how)

    # ------------------------------------------------------------ operators
    def forward(self, x):
        """y = k2y(xx2k(x2xx(x)))  (nufft/_nufft_class_methods_cpu.py:168-179)."""
        return self._call(self._lib.nufft_forward, x, 'x', 'y', 'forward')

    def adjoint(self, y):
        """x = xx2x(k2xx(y2k(y))), scaled by 1/prod(Kd) (:181-193)."""
        return self._call(self._lib.nufft_adjoint, y, 'y', 'x', 'adjoint')

    def selfadjoint(self, x):
        """adjoint(forward(x)) (:201-214)."""
        return self._call(self._lib.nufft_selfadjoint, x, 'x', 'x', 'selfadjoint')

    def x2xx(self, x):
        return self._call(self._lib.nufft_x2xx, x, 'x', 'x', 'x2xx')

    def xx2x(self, xx):
        return self._call(self._lib.nufft_xx2x, xx, 'x', 'x', 'xx2x')

    def xx2k(self, xx):
        return self._call(self._lib.nufft_xx2k, xx, 'x', 'k', 'xx2k')

    def k2xx(self, k):
        return self._call(self._lib.nufft_k2xx, k, 'k', 'x', 'k2xx')

    def k2y(self, k):
        return self._call(self._lib.nufft_k2y, k, 'k', 'y', 'k2y')

    def y2k(self, y):
        return self._call(self._lib.nufft_y2k, y, 'y', 'k', 'y2k')

    def k2y2k(self, k):
        return self._call(self._lib.nufft_k2y2k, k, 'k', 'k', 'k2y2k')

    # ---- many host arrays, copies overlapped with the transforms
    _STAGES = {'forward': ('x', 'y'), 'adjoint': ('y', 'x'), 'selfadjoint': ('x', 'x'),
               'x2xx': ('x', 'x'), 'xx2x': ('x', 'x'), 'xx2k': ('x', 'k'), 'k2xx': ('k', 'x'),
               'k2y': ('k', 'y'), 'y2k': ('y', 'k'), 'k2y2k': ('k', 'k')}

    def run_many(self, jobs, depth=2, out=None, lanes=1):
        """Apply a sequence of operators to host arrays, with the host link
        busy while the GPU transforms.

        jobs: iterable of (name, array): name one of forward, adjoint,
        selfadjoint, x2xx, xx2x, xx2k, k2xx, k2y, y2k, k2y2k; array a CPU
        tensor or numpy array of that operator's input shape (pinned CPU
        tensors are copied without staging).  Inputs are copied to the
        device on an upload stream, the operators run in order on the
        current stream, and results are copied back on a download stream
        into pinned CPU tensors, so the copies of job i+1's input and job
        i-1's result overlap job i's transform; `depth` jobs' device buffers
        rotate.  With ``lanes`` = L > 1, job i runs on lane i mod L: lane 0
        is this operator on the current stream, the others are twin
        operators of the same points (made on first use and kept; each holds
        its own plan tables and scratch) on streams of their own, so that
        the transforms of independent jobs overlap on the GPU.  Returns the
        results in order (written into `out`, a list of pinned complex64
        CPU tensors of the results' shapes, when given).  Each result equals
        that of calling the method alone (bitwise on deterministic plans).
        """
        torch = _torch()
        if self._plan is None:
            raise RuntimeError('plan() has not been called')
        if depth < 1:
            raise ValueError('depth must be at least 1')
        if lanes < 1:
            raise ValueError('lanes must be at least 1')
        todo = []
        for name, a in jobs:
            if name not in self._STAGES:
                raise ValueError(f'unknown operator {name!r}')
            kin, kout = self._STAGES[name]
            if isinstance(a, torch.Tensor):
                if a.is_cuda:
                    raise ValueError('run_many takes host arrays; call the method on device tensors')
                h = a.to(torch.complex64).contiguous()
            else:
                h = torch.from_numpy(numpy.ascontiguousarray(a, dtype=numpy.complex64))
            if tuple(h.shape) != self._shape(kin):
                raise ValueError(f'{name}: expected shape {self._shape(kin)}, got {tuple(h.shape)}')
            todo.append((name, h if h.is_pinned() else h.pin_memory(), kin, kout))
        if out is not None:
            out = list(out)
            if len(out) != len(todo):
                raise ValueError(f'out: {len(out)} tensors for {len(todo)} jobs')
            for (name, _, _, kout), o in zip(todo, out):
                if (not isinstance(o, torch.Tensor) or o.is_cuda or not o.is_pinned()
                        or o.dtype != torch.complex64 or not o.is_contiguous()
                        or tuple(o.shape) != self._shape(kout)):
                    raise ValueError(f'out: {name} needs a pinned contiguous complex64 CPU '
                                     f'tensor of shape {self._shape(kout)}')
        lanes = max(1, min(lanes, len(todo)))
        dev = self.device
        comp = torch.cuda.current_stream(dev)
        if getattr(self, '_copy_streams', None) is None:   # made once per operator
            self._copy_streams = (torch.cuda.Stream(dev), torch.cuda.Stream(dev))
        up, down = self._copy_streams
        with torch.cuda.device(dev):
            while len(self._twins) < lanes - 1:
                self._twins.append(self._twin())
            if len(self._lane_streams) < lanes - 1:
                self._lane_streams = [torch.cuda.Stream(dev) for _ in range(lanes - 1)]
            ops = [self] + self._twins[:lanes - 1]
            streams = [comp] + self._lane_streams[:lanes - 1]
            for s in streams[1:]:
                s.wait_stream(comp)
            bufs = {}
            freed_in = {}     # compute of the (lane, slot)'s last job done
            freed_out = {}    # download of the (lane, slot)'s last result done
            outs = []
            for i, (name, h, kin, kout) in enumerate(todo):
                ln = i % lanes
                s = (ln, (i // lanes) % depth)
                cs = streams[ln]
                din = bufs.get((s, 'in', kin))
                if din is None:
                    din = bufs[(s, 'in', kin)] = self._empty(kin)
                dout = bufs.get((s, 'out', kout))
                if dout is None:
                    dout = bufs[(s, 'out', kout)] = self._empty(kout)
                with torch.cuda.stream(up):
                    if s in freed_in:
                        up.wait_event(freed_in[s])
                    din.copy_(h, non_blocking=True)
                    ev_up = torch.cuda.Event()
                    ev_up.record(up)
                cs.wait_event(ev_up)
                if s in freed_out:
                    cs.wait_event(freed_out[s])
                fn = getattr(self._lib, 'nufft_' + name)
                _lib.check(fn(ops[ln]._plan, c_void_p(din.data_ptr()), c_void_p(dout.data_ptr()),
                              c_void_p(cs.cuda_stream)), name)
                ev_comp = torch.cuda.Event()
                ev_comp.record(cs)
                freed_in[s] = ev_comp
                o = (out[i] if out is not None else
                     torch.empty(self._shape(kout), dtype=torch.complex64, pin_memory=True))
                with torch.cuda.stream(down):
                    down.wait_event(ev_comp)
                    o.copy_(dout, non_blocking=True)
                    ev_down = torch.cuda.Event()
                    ev_down.record(down)
                freed_out[s] = ev_down
                outs.append(o)
            down.synchronize()
            comp.wait_stream(up)      # the buffers die with this call
            for s in streams[1:]:
                comp.wait_stream(s)
        return outs

    # ---- single-image FFT stages (nufft/_nufft_class_methods_cpu.py:251-264, 332-344)
    def _single_image_plan(self):
        """This plan when it is one coil and one instance; otherwise a
        point-free single-coil plan of the same Nd/Kd/Jd (kept), whose FFT
        stages transform one Nd image."""
        if self.B == 1 and self.ninst == 1:
            return self
        one = getattr(self, '_one2one', None)
        if one is None or one.Nd != self.Nd or one.Kd != self.Kd or one.Jd != self.Jd:
            one = NUFFT(self.device)
            one.plan(numpy.zeros((0, self.ndims)), self.Nd, self.Kd, self.Jd)
            self._one2one = one
        return one

    def xx2k_one2one(self, xx):
        """Zero-pad one Nd image into Kd and FFT it (no scaling), whatever the
        plan's batch: Nd -> Kd (nufft/__init__.py:722-724)."""
        return self._single_image_plan().xx2k(xx)

    def k2xx_one2one(self, k):
        """Inverse FFT of one Kd spectrum and crop to Nd (no scaling): Kd ->
        Nd (nufft/__init__.py:718-720)."""
        return self._single_image_plan().k2xx(k)

    # ---- SENSE coil operators (deprecated reference class, linalg/nufft_cpu.py:163-203)
    def set_sense(self, coil_profile):
        """Coil sensitivities of shape Nd + (batch,) for forward_one2many /
        adjoint_many2one."""
        torch = _torch()
        if self.batch is None:
            raise ValueError('set_sense needs a plan with batch = number of coils')
        shape = self.Nd + (self.batch,)
        if tuple(coil_profile.shape) != shape:
            raise ValueError(f'coil_profile must have shape {shape}')
        if isinstance(coil_profile, torch.Tensor) and coil_profile.is_cuda:
            m = coil_profile.to(self.device, torch.complex64).contiguous()
            self._maps = m
            ptr, on_dev = m.data_ptr(), 1
        else:
            m = numpy.ascontiguousarray(numpy.asarray(coil_profile), dtype=numpy.complex64)
            self._maps = m
            ptr, on_dev = m.ctypes.data, 0
        with torch.cuda.device(self.device):
            _lib.check(self._lib.nufft_set_sense(self._plan, c_void_p(ptr), on_dev, self._stream()),
                       'set_sense')

    def reset_sense(self):
        """All-ones coil maps (the reference's reset_sense)."""
        self.set_sense(numpy.ones(self.Nd + (self.batch,), dtype=numpy.complex64))

    def forward_one2many(self, x):
        """y = forward(x * coil maps): image Nd -> samples (M, batch)."""
        torch = _torch()
        lead = (self.ninst,) if self.ninst > 1 else ()
        if self.batch is None or self.ninst > 1:
            raise ValueError('forward_one2many needs a single-instance batch plan')
        if isinstance(x, torch.Tensor):
            if tuple(x.shape) != self.Nd:
                raise ValueError(f'expected shape {self.Nd}')
            d = x.to(self.device, torch.complex64).contiguous()
            how = ('cuda', None) if x.is_cuda else ('cpu', x.is_pinned())
        else:
            a = numpy.ascontiguousarray(numpy.asarray(x), dtype=numpy.complex64)
            if a.shape != self.Nd:
                raise ValueError(f'expected shape {self.Nd}')
            d, how = torch.from_numpy(a).to(self.device), ('numpy', None)
        out = self._empty('y')
        with torch.cuda.device(self.device):
            _lib.check(self._lib.nufft_forward_one2many(self._plan, c_void_p(d.data_ptr()),
                                                        c_void_p(out.data_ptr()), self._stream()),
                       'forward_one2many')
        return self._out(out, how)

    def adjoint_many2one(self, y):
        """x = mean over coils of conj(maps) * adjoint(y): (M, batch) -> Nd."""
        torch = _torch()
        if self.batch is None or self.ninst > 1:
            raise ValueError('adjoint_many2one needs a single-instance batch plan')
        d, how = self._in(y, 'y')
        out = torch.empty(self.Nd, dtype=torch.complex64, device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.nufft_adjoint_many2one(self._plan, c_void_p(d.data_ptr()),
                                                        c_void_p(out.data_ptr()), self._stream()),
                       'adjoint_many2one')
        return self._out(out, how)

    def selfadjoint_one2many2one(self, x):
        return self.adjoint_many2one(self.forward_one2many(x))

    def forward_dom(self, x):
        """d y / d om: an (ndim, M[, batch]) array with
        dy[d, m] = sum_n x_n (-i (n_d - N_d/2)) exp(-i om_m . (n - N/2)),
        computed as the NUFFT of (-i (n_d - N_d/2)) x."""
        torch = _torch()
        d, how = self._in(x, 'x')
        out = torch.empty((self.ndims,) + self._shape('y'), dtype=torch.complex64,
                          device=self.device)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.nufft_forward_dom(self._plan, c_void_p(d.data_ptr()),
                                                   c_void_p(out.data_ptr()), self._stream()),
                       'forward_dom')
        return self._out(out, how)

    def _solve_l1tvols(self, y, maxiter=None, rho=None, **kwargs):
        """solve(y, 'L1TVOLS', maxiter, rho) (L1TVOLS, linalg/solve_cpu.py:42-163):
        split-Bregman L1-TV least squares, mu = 1, lambda = rho, x0 = 0."""
        if kwargs:
            raise TypeError('L1TVOLS() got unexpected keyword arguments ' + ', '.join(kwargs))
        if maxiter is None or rho is None:
            raise TypeError("L1TVOLS() needs maxiter and rho")
        if self.batch is not None or self.ninst > 1:
            raise NotImplementedError('L1TVOLS runs on single-coil, single-instance plans')
        torch = _torch()
        d, how = self._in(y, 'y')
        out = self._empty('x')
        with torch.cuda.device(self.device):
            _lib.check(self._lib.nufft_solve_l1tvols(self._plan, c_void_p(d.data_ptr()),
                                                     c_void_p(out.data_ptr()), int(maxiter),
                                                     float(rho), self._stream()), 'solve')
        return self._out(out, how)

    def solve(self, y, solver=None, *args, **kwargs):
        """solve(y, 'cg', maxiter=...) (linalg/solve_cpu.py:256-288 via
        nufft/_nufft_class_methods_cpu.py:150-166): CG on the k-space normal
        operator, x0 = 0, scipy's rtol/atol stopping rule, then k2xx(k)/sn.
        'L1TVOLS' runs in the library (nufft_solve_l1tvols); 'dc', 'lsqr',
        'lsmr', 'bicg', 'bicgstab', 'gmres' and 'lgmres' are in
        ``pynufft_gb300.solvers``."""
        if solver is None:
            raise ValueError('solver must be given, e.g. solve(y, "cg", maxiter=20)')
        if solver == 'L1TVOLS':
            return self._solve_l1tvols(y, *args, **kwargs)
        if solver != 'cg':
            from . import solvers
            return solvers.solve(self, y, solver, *args, **kwargs)
        maxiter = kwargs.pop('maxiter', args[0] if args else None)
        rtol = kwargs.pop('rtol', kwargs.pop('tol', 1e-5))
        atol = kwargs.pop('atol', 0.0)
        return_info = kwargs.pop('return_info', False)
        torch = _torch()
        d, how = self._in(y, 'y')
        out = self._empty('x')
        it = c_int(0)
        with torch.cuda.device(self.device):
            _lib.check(self._lib.nufft_solve_cg(self._plan, c_void_p(d.data_ptr()),
                                                c_void_p(out.data_ptr()),
                                                -1 if maxiter is None else int(maxiter),
                                                float(rtol), float(atol),
                                                ctypes.byref(it) if return_info else None,
                                                self._stream()), 'solve')
        x = self._out(out, how)
        return (x, it.value) if return_info else x
