"""Host-side mirror of the linearised 3D implicit driver (src/impdrv3d.f90).

:class:`ImpDrv3D` owns one device context of the C ABI (``lns_ctx3d_*`` in
``include/lns3d_gb300.h``): the deck values, the metrics, the frozen
operators built on the GPU from the mean flow (``genmtrx(vm, kz, vm)``,
src/lns3d.f90:149), the time step (src/temporal.f90) and the LHS factors
(formed and factored at the first step, src/impdrv3d.f90:229-319).

The disturbance ``v`` is the Fortran array ``v(5,nx,ny)`` complex*16: a numpy
complex128 array (host memory; the call stages it, like the Fortran call) or
a CUDA torch complex128 tensor (device memory; enqueued on torch's current
stream).  Every call runs the sm_103a kernels of ``lib/liblns3d_gb300.so``;
there is no CPU fallback.
"""
import ctypes

import numpy as np

from ._lib import Params3D, check, lib

FP64, MIXED = 0, 1
FIELDS = {"Ah": 0, "Bh": 1, "Dh": 2, "Dhi": 3, "Vh11": 4, "Vh12": 5, "Vh22": 6, "ABhi": 7, "dtl": 8}
METRICS = ("m1", "m2", "n1", "n2", "m11", "m12", "m22", "n11", "n12", "n22")


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _stream():
    import torch

    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class ImpDrv3D:
    """One linearised single-mode ADI problem resident on the current GPU.

    params: dict with the deck values nx, ny, dxi, deta, Ma, Re, Pr, gamma,
    omega, kz (beta), alfa, xper, yper, navier, wall, wallt, top, optx, opty,
    plus cflmax, dtmax, loctime; metrics: dict of the ten (nx, ny) arrays;
    vm: (5, nx, ny) mean flow.  precision: FP64 (reference arithmetic) or
    MIXED (FP32 scaled LHS factors and sweeps, FP64 RHS, residual and
    update).  impl: time scheme, 1 backward Euler, 2 two-step backward
    (backward Euler for the context's first step), 3 midpoint
    (src/impdrv3d.f90:130-199).  ispg, spg, spg2: the sponge (0 none, 1 spg, > 4
    spg + spg2; src/lrhs3d.f90:220-240), spg and spg2 (nx, ny) arrays.
    eps_e, buff: explicit smoother and implicit damping (src/smoother3d.f90),
    buff (nx, ny) or None for the reference's default of ones.  ispg 2, 3,
    the forced top (params top = 1) and, with xper = 0, the wave planes
    (left 1 or 5, right 5) take the x coordinates x (nx, ny), x0 and wamp
    (nx; None: ones); ispg 4 the complex target cvic (5, nx, ny).
    wall = 3 (the bump) takes u1w, u2w, u3w, tw, twp as bump, complex (5, nx).
    row_pairs: FP64 periodic lines with an odd band advance their recurrences
    two rows per step (lns_ctx3d_set_row_pairs); False keeps them row by
    row, as a batch does.
    """

    def __init__(self, params, metrics, vm, cflmax=1.0, dtmax=1e30, loctime=1, precision=FP64,
                 impl=1, ispg=0, spg=None, spg2=None, eps_e=0.0, buff=None, x=None, x0=0.0, wamp=None,
                 cvic=None, bump=None, row_pairs=True, profile=None, lalpha=0j):
        """profile: with xper = 0 and left 4, the eigenfunction of the xi
        planes, complex (5, ny) (the inflow.dat columns); lalpha its complex
        streamwise wavenumber for right 4, whose column nx holds profile *
        exp(i lalpha x(nx, j)) (x needed)."""
        p = params
        self.nx, self.ny = int(p["nx"]), int(p["ny"])
        self.precision = precision
        prm = Params3D(nx=self.nx, ny=self.ny, dxi=p["dxi"], deta=p["deta"], Ma=p["Ma"], Re=p["Re"], Pr=p["Pr"],
                       gamma=p["gamma"], gamma1=p.get("gamma1", 0.0), omega=p["omega"], beta=p["kz"],
                       alfa=p["alfa"], cflmax=cflmax, dtmax=dtmax, loctime=loctime, xper=p["xper"], yper=p["yper"],
                       navier=p["navier"], wall=p["wall"], wallt=p["wallt"], top=p["top"], optx=p["optx"],
                       opty=p["opty"], precision=precision, impl=impl, ispg=ispg, eps_e=eps_e,
                       left=p.get("left", -1), right=p.get("right", -1))
        self._ctx = ctypes.c_void_p()
        check(lib().lns_ctx3d_create(ctypes.byref(prm), ctypes.byref(self._ctx)), "lns_ctx3d_create")
        if not row_pairs:
            check(lib().lns_ctx3d_set_row_pairs(self._ctx, 0), "lns_ctx3d_set_row_pairs")
        m = np.empty((self.nx, self.ny, 10), order="F")
        for k, name in enumerate(METRICS):
            m[:, :, k] = metrics[name]
        check(lib().lns_upload_metrics3d(self._ctx, ctypes.c_void_p(m.ctypes.data)), "lns_upload_metrics3d")
        if ispg:
            s1 = np.asfortranarray(spg, dtype=np.float64)
            s2 = np.asfortranarray(spg2, dtype=np.float64) if spg2 is not None else None
            check(lib().lns_upload_sponge3d(self._ctx, ctypes.c_void_p(s1.ctypes.data),
                                            ctypes.c_void_p(s2.ctypes.data) if s2 is not None else None),
                  "lns_upload_sponge3d")
        waves = not int(p["xper"]) and (int(p.get("left", -1)) in (1, 5) or int(p.get("right", -1)) == 5)
        if ispg in (2, 3) or int(p["top"]) == 1 or waves:
            xx = np.asfortranarray(x, dtype=np.float64)
            wa = np.ascontiguousarray(wamp, dtype=np.float64) if wamp is not None else None
            check(lib().lns_upload_inflow3d(self._ctx, ctypes.c_void_p(xx.ctypes.data),
                                            ctypes.c_void_p(wa.ctypes.data) if wa is not None else None, x0),
                  "lns_upload_inflow3d")
        if not int(p["xper"]) and int(p.get("left", -1)) == 4:
            pr = np.asfortranarray(profile, dtype=np.complex128)
            assert pr.shape == (5, self.ny)
            xr = np.ascontiguousarray(np.asarray(x)[-1, :], dtype=np.float64) if x is not None else None
            check(lib().lns_upload_profile3d(self._ctx, ctypes.c_void_p(pr.ctypes.data),
                                             ctypes.c_void_p(xr.ctypes.data) if xr is not None else None,
                                             complex(lalpha).real, complex(lalpha).imag), "lns_upload_profile3d")
        if ispg == 4:
            cv = np.asfortranarray(cvic, dtype=np.complex128)
            check(lib().lns_upload_sponge_target3d(self._ctx, ctypes.c_void_p(cv.ctypes.data)),
                  "lns_upload_sponge_target3d")
        if int(p["wall"]) == 3:
            bb = np.asfortranarray(bump, dtype=np.complex128)
            check(lib().lns_upload_bump3d(self._ctx, ctypes.c_void_p(bb.ctypes.data)), "lns_upload_bump3d")
        if eps_e and buff is not None:
            b = np.asfortranarray(buff, dtype=np.float64)
            check(lib().lns_upload_buffer3d(self._ctx, ctypes.c_void_p(b.ctypes.data)), "lns_upload_buffer3d")
        self.set_mean(vm)

    def set_mean(self, vm):
        """Upload a mean flow; rebuild the operators and time step on the GPU."""
        vm = np.asfortranarray(vm, dtype=np.float64)
        assert vm.shape == (5, self.nx, self.ny)
        cfl = ctypes.c_double()
        check(lib().lns_upload_mean3d(self._ctx, ctypes.c_void_p(vm.ctypes.data), ctypes.byref(cfl)),
              "lns_upload_mean3d")
        self.cfl = cfl.value

    @property
    def device_bytes(self):
        return lib().lns_ctx3d_bytes(self._ctx)

    def _check_v(self, v, name="v"):
        n = 5 * self.nx * self.ny
        if _is_torch(v):
            import torch

            if v.dtype != torch.complex128 or not v.is_cuda or not v.is_contiguous() or v.numel() != n:
                raise ValueError("%s must be a contiguous CUDA complex128 tensor of %d elements" % (name, n))
            return ctypes.c_void_p(v.data_ptr()), True
        if not isinstance(v, np.ndarray) or v.dtype != np.complex128 or v.size != n:
            raise ValueError("%s must be a complex128 array of shape (5, nx, ny)" % name)
        if not v.flags.f_contiguous:
            raise ValueError("%s must be Fortran-ordered (5, nx, ny)" % name)
        return ctypes.c_void_p(v.ctypes.data), False

    def itrbc(self, v):
        """itrBC3D on v in place: the reference applies it once before the
        step loop (src/impdrv3d.f90:125-126).  A host v is staged through
        the device."""
        pv, dev = self._check_v(v)
        if dev:
            check(lib().lns_itrbc3d_dev(self._ctx, pv, _stream()), "lns_itrbc3d_dev")
            return
        import torch

        t = torch.from_numpy(v.ravel(order="F")).cuda()
        check(lib().lns_itrbc3d_dev(self._ctx, ctypes.c_void_p(t.data_ptr()), _stream()), "lns_itrbc3d_dev")
        v[...] = t.cpu().numpy().reshape(v.shape, order="F")

    def step(self, v, nsteps=1, niter=1, totres=None):
        """Advance v in place by nsteps implicit steps of niter correctors.

        Host v: returns a numpy array of the per-step residuals.  Device v:
        `totres` may be a CUDA float64 tensor of nsteps entries that receives
        them; returns None (asynchronous)."""
        pv, dev = self._check_v(v)
        if dev:
            pt = ctypes.c_void_p(totres.data_ptr()) if totres is not None else None
            check(lib().lns_step3d_dev(self._ctx, pv, nsteps, niter, pt, _stream()), "lns_step3d_dev")
            return None
        res = np.zeros(max(nsteps, 1))
        check(lib().lns_step3d(self._ctx, pv, nsteps, niter, ctypes.c_void_p(res.ctypes.data)), "lns_step3d")
        return res[:nsteps]

    def rhs(self, v, vold, r, totres=None):
        """r = rhsBC3D(rbe3D(lrhs3D(v))) on device tensors; totres: 1-element tensor."""
        pv, _ = self._check_v(v)
        po, _ = self._check_v(vold, "vold")
        pr, _ = self._check_v(r, "r")
        pt = ctypes.c_void_p(totres.data_ptr()) if totres is not None else None
        check(lib().lns_rhs3d_dev(self._ctx, pv, po, pr, pt, _stream()), "lns_rhs3d_dev")

    def lhs(self, direction, mat):
        """Unfactored LHS of the xi (1) or eta (2) sweep into a device tensor of 125 nx ny complex128."""
        if mat.numel() != 125 * self.nx * self.ny or not mat.is_cuda:
            raise ValueError("mat must be a CUDA tensor of 125*nx*ny complex128 entries")
        check(lib().lns_lhs3d_dev(self._ctx, direction, ctypes.c_void_p(mat.data_ptr()), _stream()), "lns_lhs3d_dev")

    def field(self, name):
        """A frozen field in the reference layout (numpy, Fortran order)."""
        shape = {0: (5, 5), 1: (5, 5), 2: (5, 5), 3: (5, 5), 8: ()}.get(FIELDS[name], (6,))
        out = np.zeros(shape + (self.nx, self.ny), order="F")
        check(lib().lns_get_field3d(self._ctx, FIELDS[name], ctypes.c_void_p(out.ctypes.data)), "lns_get_field3d")
        return out

    def profile(self, on=True):
        """Start (or stop) recording per-phase CUDA events of every corrector."""
        check(lib().lns_ctx3d_profile(self._ctx, 1 if on else 0), "lns_ctx3d_profile")

    SEGMENTS = ("rhs", "x_scale", "x_fwd", "x_bwd", "x_fill", "y_scale", "y_fwd", "y_bwd", "update")

    def profile_read(self):
        """Summed milliseconds per kernel segment (SEGMENTS) and per phase
        (rhs, xsweep, ysweep, update), and the number of correctors recorded
        since profiling started."""
        ms = np.zeros(len(self.SEGMENTS))
        n = ctypes.c_int32()
        check(lib().lns_ctx3d_profile_read(self._ctx, ctypes.c_void_p(ms.ctypes.data), ctypes.byref(n)),
              "lns_ctx3d_profile_read")
        seg = dict(zip(self.SEGMENTS, ms.tolist()))
        phases = {"rhs": seg["rhs"], "xsweep": sum(seg[k] for k in ("x_scale", "x_fwd", "x_fill", "x_bwd")),
                  "ysweep": sum(seg[k] for k in ("y_scale", "y_fwd", "y_bwd")), "update": seg["update"]}
        return phases, n.value, seg

    def close(self):
        if self._ctx:
            lib().lns_ctx3d_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch3D:
    """Many linearised problems advanced together (lns_batch3d_* of the C ABI).

    problems: list of dicts with keys params, metrics, vm, v (as for
    ImpDrv3D / lns3d_gb300.cases.shear_layer).  Every phase of a step is one
    launch for all problems and the step is replayed as a CUDA graph; each
    problem's result equals its own ImpDrv3D run.
    """

    def __init__(self, problems, cflmax=1.0, dtmax=1e30, loctime=1, precision=FP64):
        self.P = len(problems)
        self.shapes = []
        arr = (Params3D * self.P)()
        for k, pr in enumerate(problems):
            p = pr["params"]
            arr[k] = Params3D(nx=p["nx"], ny=p["ny"], dxi=p["dxi"], deta=p["deta"], Ma=p["Ma"], Re=p["Re"],
                              Pr=p["Pr"], gamma=p["gamma"], gamma1=p.get("gamma1", 0.0), omega=p["omega"],
                              beta=p["kz"], alfa=p["alfa"], cflmax=cflmax, dtmax=dtmax, loctime=loctime,
                              xper=p["xper"], yper=p["yper"], navier=p["navier"], wall=p["wall"], wallt=p["wallt"],
                              top=p["top"], optx=p["optx"], opty=p["opty"], precision=precision)
            self.shapes.append((5, int(p["nx"]), int(p["ny"])))
        self._b = ctypes.c_void_p()
        check(lib().lns_batch3d_create(self.P, arr, ctypes.byref(self._b)), "lns_batch3d_create")
        for k, pr in enumerate(problems):
            nx, ny = self.shapes[k][1:]
            m = np.empty((nx, ny, 10), order="F")
            for i, name in enumerate(METRICS):
                m[:, :, i] = pr["metrics"][name]
            vm = np.asfortranarray(pr["vm"], dtype=np.float64)
            v = np.asfortranarray(pr["v"], dtype=np.complex128)
            check(lib().lns_batch3d_upload(self._b, k, ctypes.c_void_p(m.ctypes.data), ctypes.c_void_p(vm.ctypes.data),
                                           ctypes.c_void_p(v.ctypes.data)), "lns_batch3d_upload")

    @property
    def device_bytes(self):
        return lib().lns_batch3d_bytes(self._b)

    def tune(self, niter=1):
        w = ctypes.c_int32()
        check(lib().lns_batch3d_tune(self._b, niter, ctypes.byref(w)), "lns_batch3d_tune")
        return w.value

    def run(self, max_steps, tol=0.0, niter=1, check_every=25):
        """Steps every problem until its residual <= tol (or max_steps);
        returns (steps to tol per problem, -1 if not reached; final residuals)."""
        steps = np.zeros(self.P, dtype=np.int32)
        res = np.zeros(self.P)
        check(lib().lns_batch3d_run(self._b, max_steps, niter, tol, check_every, ctypes.c_void_p(steps.ctypes.data),
                                    ctypes.c_void_p(res.ctypes.data)), "lns_batch3d_run")
        return steps, res

    def state(self, k):
        v = np.zeros(self.shapes[k], np.complex128, order="F")
        check(lib().lns_batch3d_get_state(self._b, k, ctypes.c_void_p(v.ctypes.data)), "lns_batch3d_get_state")
        return v

    def close(self):
        if self._b:
            lib().lns_batch3d_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


REQ_STATES = {1: "queued", 2: "running", 3: "done", 4: "stopped", 5: "failed"}


class Server3D:
    """Continuous batching of linearised solves (lns_server3d_* of the C ABI).

    Requests are submitted at any time; each tick admits what fits in the
    device-memory budget and the free slots, advances every running request
    by nsteps batched steps, and retires the ones whose residual reached
    their tolerance (their state is the one that met it) or that ran out of
    steps.  A request's result does not depend on the other requests.
    """

    def __init__(self, budget_bytes, max_slots=64, precision=MIXED, niter=1):
        self.precision = precision
        self._s = ctypes.c_void_p()
        check(lib().lns_server3d_create(ctypes.c_size_t(int(budget_bytes)), max_slots, precision, niter,
                                        ctypes.byref(self._s)), "lns_server3d_create")
        self._shape = {}

    def submit(self, problem, tol=1e-10, max_steps=2000, cflmax=1.0, dtmax=1e30, loctime=1):
        p = problem["params"]
        prm = Params3D(nx=p["nx"], ny=p["ny"], dxi=p["dxi"], deta=p["deta"], Ma=p["Ma"], Re=p["Re"], Pr=p["Pr"],
                       gamma=p["gamma"], gamma1=p.get("gamma1", 0.0), omega=p["omega"], beta=p["kz"],
                       alfa=p["alfa"], cflmax=cflmax, dtmax=dtmax, loctime=loctime, xper=p["xper"], yper=p["yper"],
                       navier=p["navier"], wall=p["wall"], wallt=p["wallt"], top=p["top"], optx=p["optx"],
                       opty=p["opty"], precision=self.precision)
        nx, ny = int(p["nx"]), int(p["ny"])
        m = np.empty((nx, ny, 10), order="F")
        for i, name in enumerate(METRICS):
            m[:, :, i] = problem["metrics"][name]
        vm = np.asfortranarray(problem["vm"], dtype=np.float64)
        v = np.asfortranarray(problem["v"], dtype=np.complex128)
        rid = ctypes.c_int64()
        check(lib().lns_server3d_submit(self._s, ctypes.byref(prm), ctypes.c_void_p(m.ctypes.data),
                                        ctypes.c_void_p(vm.ctypes.data), ctypes.c_void_p(v.ctypes.data), tol,
                                        max_steps, ctypes.byref(rid)), "lns_server3d_submit")
        self._shape[rid.value] = (5, nx, ny)
        return rid.value

    def tick(self, nsteps=25):
        run, que = ctypes.c_int32(), ctypes.c_int32()
        check(lib().lns_server3d_tick(self._s, nsteps, ctypes.byref(run), ctypes.byref(que)), "lns_server3d_tick")
        return run.value, que.value

    def poll(self, rid):
        st, steps, res, lat = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_double(), ctypes.c_double()
        check(lib().lns_server3d_poll(self._s, rid, ctypes.byref(st), ctypes.byref(steps), ctypes.byref(res),
                                      ctypes.byref(lat)), "lns_server3d_poll")
        return {"state": REQ_STATES.get(st.value, st.value), "steps": steps.value, "res": res.value,
                "latency_s": lat.value}

    def fetch(self, rid):
        v = np.zeros(self._shape.pop(rid), np.complex128, order="F")
        check(lib().lns_server3d_fetch(self._s, rid, ctypes.c_void_p(v.ctypes.data)), "lns_server3d_fetch")
        return v

    @property
    def bytes_in_use(self):
        return lib().lns_server3d_bytes_in_use(self._s)

    @property
    def graph_captures(self):
        return lib().lns_server3d_graph_captures(self._s)

    def close(self):
        if self._s:
            lib().lns_server3d_destroy(self._s)
            self._s = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ImpDrvLin2D:
    """The linearised 2D implicit step (src/impdrv.f90 with linear = 1,
    src/lrhs.f90) on the current GPU: real fields v (5, nx, ny).

    params: as ImpDrv3D's, with kz = 0 and omega = 0 (a deck with Lz = 0);
    metrics: the ten (nx, ny) arrays; vm: (5, nx, ny) mean flow.  The
    context runs the single-mode machinery at kz = omega = 0.  nbl: the
    &extras namelist's nbl for the nonreflecting planes (left 1, right 1),
    which act on rows j > nbl."""

    def __init__(self, params, metrics, vm, cflmax=1.0, dtmax=1e30, loctime=1, impl=1, ispg=0, eps_e=0.0, nbl=0):
        p = params
        if p.get("kz", 0.0) != 0.0 or p.get("omega", 0.0) != 0.0:
            raise ValueError("a 2D linear run has kz = 0 and omega = 0")
        self.nx, self.ny = int(p["nx"]), int(p["ny"])
        prm = Params3D(nx=self.nx, ny=self.ny, dxi=p["dxi"], deta=p["deta"], Ma=p["Ma"], Re=p["Re"], Pr=p["Pr"],
                       gamma=p["gamma"], gamma1=p.get("gamma1", 0.0), omega=0.0, beta=0.0, alfa=p["alfa"],
                       cflmax=cflmax, dtmax=dtmax, loctime=loctime, xper=p["xper"], yper=p["yper"],
                       navier=p["navier"], wall=p["wall"], wallt=p["wallt"], top=p["top"], optx=p["optx"],
                       opty=p["opty"], precision=FP64, impl=impl, ispg=ispg, eps_e=eps_e,
                       left=p.get("left", -1), right=p.get("right", -1))
        self._ctx = ctypes.c_void_p()
        check(lib().lns_lin2d_create(ctypes.byref(prm), ctypes.byref(self._ctx)), "lns_lin2d_create")
        if nbl:
            check(lib().lns_lin2d_set_nbl(self._ctx, int(nbl)), "lns_lin2d_set_nbl")
        m = np.empty((self.nx, self.ny, 10), order="F")
        for k, name in enumerate(METRICS):
            m[:, :, k] = metrics[name]
        check(lib().lns_upload_metrics_lin2d(self._ctx, ctypes.c_void_p(m.ctypes.data)), "lns_upload_metrics_lin2d")
        vm = np.asfortranarray(vm, dtype=np.float64)
        cfl = ctypes.c_double()
        check(lib().lns_upload_mean_lin2d(self._ctx, ctypes.c_void_p(vm.ctypes.data), ctypes.byref(cfl)),
              "lns_upload_mean_lin2d")
        self.cfl = cfl.value

    def _check(self, v):
        if not isinstance(v, np.ndarray) or v.dtype != np.float64 or v.shape != (5, self.nx, self.ny) \
                or not v.flags.f_contiguous:
            raise ValueError("v must be a Fortran-ordered float64 array of shape (5, nx, ny)")

    def itrbc(self, v):
        """itrBC on v in place (the call before the step loop, src/impdrv.f90:160)."""
        import torch

        self._check(v)
        t = torch.from_numpy(v.ravel(order="F")).cuda()
        check(lib().lns_itrbc_lin2d_dev(self._ctx, ctypes.c_void_p(t.data_ptr()), _stream()), "lns_itrbc_lin2d_dev")
        v[...] = t.cpu().numpy().reshape(v.shape, order="F")

    def step(self, v, nsteps=1, niter=1):
        """nsteps steps of niter correctors on host v in place; the per-step residuals."""
        self._check(v)
        res = np.zeros(max(nsteps, 1))
        check(lib().lns_step_lin2d(self._ctx, ctypes.c_void_p(v.ctypes.data), nsteps, niter,
                                   ctypes.c_void_p(res.ctypes.data)), "lns_step_lin2d")
        return res[:nsteps]

    def __del__(self):
        if getattr(self, "_ctx", None) and self._ctx.value:
            lib().lns_lin2d_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()
