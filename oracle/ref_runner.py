"""Run the reference's own CUDA kernels (fatbins built from the reference
sources by oracle/build_ref.py) on a GPU, replaying the launch sequence of
CudaLinearSearchAlgorithm (cuda/src/semblance/algorithm/
CudaLinearSearchAlgorithm.cu:35-324) and CudaStretchFreeAlgorithm
(CudaStretchFreeAlgorithm.cu:28-200) for one midpoint at a time.

TEST INFRASTRUCTURE ONLY: used to generate golden fixtures
(tests/golden/make_reference_golden.py) and the reference-CUDA timing.  It
uses the CUDA driver API through ctypes (libcuda.so.1) and torch for device
memory; kernels are looked up by their C++ names in the loaded module.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path
from typing import Dict, List, Optional

import numpy as np

REF_DIR = Path(__file__).resolve().parent / "_ref"
THREADS = 64  # DEFAULT_THREAD_COUNT (ComputeAlgorithm.hpp:16)


def available() -> bool:
    return (REF_DIR / "cmp_linear_search.fatbin").exists()


class Driver:
    def __init__(self):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.torch = torch
        self.cu = C.CDLL("libcuda.so.1")
        self.cu.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_void_p]
        self.cu.cuModuleGetFunctionCount.argtypes = [C.POINTER(C.c_uint), C.c_void_p]
        self.cu.cuModuleEnumerateFunctions.argtypes = [C.POINTER(C.c_void_p), C.c_uint, C.c_void_p]
        self.cu.cuFuncGetName.argtypes = [C.POINTER(C.c_char_p), C.c_void_p]
        self.cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                           C.c_uint, C.c_uint, C.c_uint, C.c_void_p,
                                           C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        self.cu.cuCtxSynchronize.argtypes = []
        self.modules: Dict[str, Dict[str, C.c_void_p]] = {}
        self._blobs = []

    def _chk(self, r, what):
        if r != 0:
            raise RuntimeError(f"CUDA driver error {r} in {what}")

    def module(self, name: str) -> Dict[str, C.c_void_p]:
        if name in self.modules:
            return self.modules[name]
        blob = (REF_DIR / f"{name}.fatbin").read_bytes()
        buf = C.create_string_buffer(blob, len(blob))
        self._blobs.append(buf)
        mod = C.c_void_p()
        self._chk(self.cu.cuModuleLoadData(C.byref(mod), buf), "cuModuleLoadData " + name)
        n = C.c_uint()
        self._chk(self.cu.cuModuleGetFunctionCount(C.byref(n), mod), "cuModuleGetFunctionCount")
        funcs = (C.c_void_p * n.value)()
        self._chk(self.cu.cuModuleEnumerateFunctions(funcs, n.value, mod),
                  "cuModuleEnumerateFunctions")
        table = {}
        for f in funcs:
            nm = C.c_char_p()
            self._chk(self.cu.cuFuncGetName(C.byref(nm), f), "cuFuncGetName")
            table[_plain_name(nm.value.decode())] = C.c_void_p(f)
        self.modules[name] = table
        return table

    def launch(self, func, grid: int, block: int, args: List):
        holders = []
        ptrs = (C.c_void_p * len(args))()
        for i, a in enumerate(args):
            holders.append(a)
            ptrs[i] = C.cast(C.pointer(a), C.c_void_p)
        self._chk(self.cu.cuLaunchKernel(func, grid, 1, 1, block, 1, 1, 0, None, ptrs, None),
                  "cuLaunchKernel")
        self._chk(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")


def _plain_name(mangled: str) -> str:
    """C++ name of an Itanium-mangled function symbol (_Z<len><name>...)."""
    if not mangled.startswith("_Z"):
        return mangled
    i = 2
    j = i
    while j < len(mangled) and mangled[j].isdigit():
        j += 1
    n = int(mangled[i:j])
    return mangled[j:j + n]


def _grid(n: int) -> int:
    # dim3 dimGrid(ceil(float(n) / float(threadCount)))
    return int(math.ceil(np.float32(n) / np.float32(THREADS)))


class ReferenceKernels:
    """The reference's CUDA kernels behind a numpy interface."""

    def __init__(self):
        self.d = Driver()
        self.torch = self.d.torch

    def _dev(self, a: np.ndarray):
        return self.torch.from_numpy(np.ascontiguousarray(a)).cuda()

    def _ptr(self, t):
        return C.c_void_p(t.data_ptr())

    def build_grid(self, model: str, lower, upper, gran) -> np.ndarray:
        """initializeParameters (CudaLinearSearchAlgorithm.cu:165-223)."""
        f32 = np.float32
        steps = [f32(f32(upper[j]) - f32(lower[j])) / f32(gran[j]) for j in range(len(gran))]
        P = int(np.prod(gran))
        npar = len(gran)
        out = self.torch.zeros(P * npar, dtype=self.torch.float32, device="cuda")
        if model == "cmp":
            k = self.d.module("cmp_linear_search")["buildParameterArrayForCommonMidPoint"]
            args = [self._ptr(out), C.c_float(lower[0]), C.c_float(steps[0]), C.c_uint(P)]
        elif model == "zocrs":
            k = self.d.module("zocrs_linear_search")[
                "buildParameterArrayForZeroOffsetCommonReflectionSurface"]
            args = [self._ptr(out)]
            for j in range(3):
                args += [C.c_float(lower[j]), C.c_float(steps[j]), C.c_uint(gran[j])]
            args += [C.c_uint(P)]
        else:
            k = self.d.module("oct_linear_search")[
                "buildParameterArrayForOffsetContinuationTrajectory"]
            args = [self._ptr(out)]
            for j in range(2):
                args += [C.c_float(lower[j]), C.c_float(steps[j]), C.c_uint(gran[j])]
            args += [C.c_uint(P)]
        self.d.launch(k, _grid(P), THREADS, args)
        return out.cpu().numpy().reshape(P, npar)

    def select(self, model: str, mid, hoff, m0: float, apm: float, h0: float, S: int,
               dt: float, cands: Optional[np.ndarray] = None) -> np.ndarray:
        """selectTracesFor* (cmp/common.cu, zocrs/common.cu, oct/linear_search.cu)."""
        n = len(mid)
        dmid = self._dev(np.asarray(mid, np.float32))
        mask = self.torch.zeros(n, dtype=self.torch.uint8, device="cuda")
        if model == "cmp":
            k = self.d.module("cmp_common")["selectTracesForCommonMidPoint"]
            args = [self._ptr(dmid), C.c_uint(n), self._ptr(mask), C.c_float(m0)]
        elif model == "zocrs":
            k = self.d.module("zocrs_common")["selectTracesForZeroOffsetCommonReflectionSurface"]
            args = [self._ptr(dmid), C.c_uint(n), self._ptr(mask), C.c_float(m0),
                    C.c_float(apm)]
        else:
            k = self.d.module("oct_linear_search")["selectTracesForOffsetContinuationTrajectory"]
            dh = self._dev(np.asarray(hoff, np.float32))
            dc = self._dev(np.asarray(cands, np.float32).ravel())
            args = [self._ptr(dmid), self._ptr(dh), self._ptr(dc), C.c_uint(len(cands)),
                    C.c_uint(n), C.c_uint(S), C.c_float(dt), C.c_float(apm), C.c_float(m0),
                    C.c_float(h0), self._ptr(mask)]
        self.d.launch(k, _grid(n), THREADS, args)
        return mask.cpu().numpy().astype(bool)

    def linear_search_midpoint(self, model: str, samples, mid, hoff, sel, m0: float, dt: float,
                               tau: int, params: np.ndarray, apm: float = 0.0,
                               h0: float = 0.0, timing: bool = False):
        """computeSemblanceAtGpuForMidpoint (CudaLinearSearchAlgorithm.cu:35-163).
        Returns (result [(2+np)][S], sembl [S][P], stack [S][P], notUsed [S*P]),
        plus the device ms of the evaluation and argmax launches if timing."""
        S = samples.shape[1]
        P = params.shape[0]
        npar = params.shape[1]
        sel = np.asarray(sel)
        n = sel.size
        w = 2 * tau + 1
        res = self.torch.zeros((2 + npar) * S, dtype=self.torch.float32, device="cuda")
        nu = self.torch.zeros(S * P, dtype=self.torch.float32, device="cuda")
        sem = self.torch.zeros(S * P, dtype=self.torch.float32, device="cuda")
        stk = self.torch.zeros(S * P, dtype=self.torch.float32, device="cuda")
        if n == 0:
            z = np.zeros(((2 + npar), S), np.float32)
            return z, np.zeros((S, P), np.float32), np.zeros((S, P), np.float32), np.zeros(S * P)
        smp = self._dev(np.ascontiguousarray(samples[sel], np.float32).ravel())
        hf = np.asarray(hoff, np.float32)[sel]
        dm = self._dev(np.asarray(mid, np.float32)[sel])
        dh = self._dev(hf)
        dh2 = self._dev((hf * hf).astype(np.float32))
        dp = self._dev(np.ascontiguousarray(params, np.float32).ravel())
        g = _grid(S * P)
        gb = _grid(S)
        e0 = self.torch.cuda.Event(enable_timing=True)
        e1 = self.torch.cuda.Event(enable_timing=True)
        e0.record()
        if model == "cmp":
            mod = self.d.module("cmp_linear_search")
            self.d.launch(mod["computeSemblancesForCommonMidPoint"], g, THREADS,
                          [self._ptr(smp), self._ptr(dh2), C.c_uint(n), C.c_uint(S),
                           C.c_float(dt), C.c_int(tau), C.c_int(w), self._ptr(dp), C.c_uint(P),
                           self._ptr(sem), self._ptr(stk)])
            best = mod["selectBestSemblancesForCommonMidPoint"]
        elif model == "zocrs":
            mod = self.d.module("zocrs_linear_search")
            self.d.launch(mod["computeSemblancesForZeroOffsetCommonReflectionSurface"], g,
                          THREADS,
                          [self._ptr(smp), self._ptr(dm), self._ptr(dh2), C.c_uint(n),
                           C.c_uint(S), C.c_float(m0), C.c_float(dt), C.c_int(tau), C.c_int(w),
                           self._ptr(dp), C.c_uint(P), self._ptr(sem), self._ptr(stk)])
            best = mod["selectBestSemblancesForZeroOffsetCommonReflectionSurface"]
        else:
            mod = self.d.module("oct_linear_search")
            self.d.launch(mod["computeSemblancesForOffsetContinuationTrajectory"], g, THREADS,
                          [self._ptr(smp), self._ptr(dm), self._ptr(dh), C.c_uint(n),
                           C.c_uint(S), C.c_float(apm), C.c_float(m0), C.c_float(h0),
                           C.c_float(dt), C.c_int(tau), C.c_int(w), self._ptr(dp), C.c_uint(P),
                           self._ptr(nu), self._ptr(sem), self._ptr(stk)])
            best = mod["selectBestSemblancesForOffsetContinuationTrajectory"]
        self.d.launch(best, gb, THREADS, [self._ptr(sem), self._ptr(stk), self._ptr(dp),
                                          C.c_uint(P), C.c_uint(S), self._ptr(res)])
        e1.record()
        self.torch.cuda.synchronize()
        out = (res.cpu().numpy().reshape(2 + npar, S), sem.cpu().numpy().reshape(S, P),
               stk.cpu().numpy().reshape(S, P), nu.cpu().numpy())
        return out + (e0.elapsed_time(e1),) if timing else out

    def stretch_free_midpoint_cmp(self, samples, hoff, sel, dt: float, tau: int,
                                  prior: np.ndarray, nmax: int = 10, timing: bool = False):
        """CudaStretchFreeAlgorithm::computeSemblanceAtGpuForMidpoint for CMP
        (the only model its CUDA path runs, CudaStretchFreeAlgorithm.cu:52-66).
        prior: [S] velocities.  Returns [3][S] (semblance, stack, n), plus the
        device ms of the evaluation and argmax launches if timing."""
        S = samples.shape[1]
        nn = 2 * nmax + 1
        sel = np.asarray(sel)
        n = sel.size
        w = 2 * tau + 1
        smp = self._dev(np.ascontiguousarray(samples[sel], np.float32).ravel())
        hf = np.asarray(hoff, np.float32)[sel]
        dh2 = self._dev((hf * hf).astype(np.float32))
        dprior = self._dev(np.asarray(prior, np.float32))
        narr = self._dev(np.arange(-nmax, nmax + 1, dtype=np.float32))
        sem = self.torch.zeros(S * nn, dtype=self.torch.float32, device="cuda")
        stk = self.torch.zeros(S * nn, dtype=self.torch.float32, device="cuda")
        res = self.torch.zeros(3 * S, dtype=self.torch.float32, device="cuda")
        mod = self.d.module("cmp_stretch_free")
        e0 = self.torch.cuda.Event(enable_timing=True)
        e1 = self.torch.cuda.Event(enable_timing=True)
        e0.record()
        self.d.launch(mod["computeSemblancesForCommonMidPoint"], _grid(S * nn), THREADS,
                      [self._ptr(smp), self._ptr(dh2), C.c_uint(n), C.c_uint(S), C.c_float(dt),
                       C.c_int(tau), C.c_int(w), self._ptr(dprior), self._ptr(narr),
                       C.c_uint(nn), self._ptr(sem), self._ptr(stk)])
        best = self.d.module("common_stretch_free")["selectBestSemblances"]
        self.d.launch(best, _grid(S), THREADS, [self._ptr(sem), self._ptr(stk), self._ptr(narr),
                                                C.c_uint(nn), C.c_uint(S), self._ptr(res)])
        e1.record()
        self.torch.cuda.synchronize()
        out = res.cpu().numpy().reshape(3, S)
        return (out, e0.elapsed_time(e1)) if timing else out

    def differential_evolution_midpoint(self, model: str, samples, mid, hoff, m0: float,
                                        dt: float, tau: int, lower, upper, pop: int, gens: int,
                                        seed: int, apm: float = 0.0, h0: float = 0.0,
                                        sel=None, operators: str = "common_differential_evolution"):
        """DifferentialEvolutionAlgorithm::computeSemblanceAndParametersForMidpoint
        (DifferentialEvolutionAlgorithm.cpp:21-81) with the kernels of
        CudaDifferentialEvolutionAlgorithm (CudaDifferentialEvolutionAlgorithm.cu
        :35-353): setupRandomSeed, startPopulations, selection, evaluation of
        the initial population, then per generation mutate, crossover, evaluate
        u, nextGeneration; selectBestIndividuals.  `seed` replaces the
        reference's srand(time(NULL)); rand().  `operators` names the fatbin of
        the DE operators (F and CR are compile-time constants there).  `sel`
        (CMP / ZO-CRS): selected trace indices (the linear-search rule); OCT
        runs the reference's DE selection on the initial population.
        Returns (result [(2+np)][S], device ms from the first evaluation to
        the selection of the best individuals, selected trace count)."""
        torch = self.torch
        S = samples.shape[1]
        npar = {"cmp": 1, "zocrs": 3, "oct": 2}[model]
        n_ind = S * pop
        w = 2 * tau + 1
        ncr = 2
        f32 = torch.float32
        x = torch.zeros(n_ind * npar, dtype=f32, device="cuda")
        u = torch.zeros_like(x)
        v = torch.zeros_like(x)
        fx = torch.zeros(n_ind * ncr, dtype=f32, device="cuda")
        fu = torch.zeros_like(fx)
        nu = torch.zeros(n_ind, dtype=f32, device="cuda")
        res = torch.zeros((2 + npar) * S, dtype=f32, device="cuda")
        dmin = self._dev(np.asarray(lower, np.float32))
        dmax = self._dev(np.asarray(upper, np.float32))
        # curandStateXORWOW is 48 bytes; 64 per state leaves room
        st = torch.zeros(n_ind * 64, dtype=torch.uint8, device="cuda")
        ops = self.d.module(operators)
        ev = self.d.module(f"{model}_differential_evolution")
        g = _grid(n_ind)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        self.d.launch(ops["setupRandomSeed"], g, THREADS,
                      [self._ptr(st), C.c_uint(seed & 0xffffffff), C.c_uint(pop), C.c_uint(S)])
        self.d.launch(ops["startPopulations"], g, THREADS,
                      [self._ptr(x), self._ptr(dmin), self._ptr(dmax), self._ptr(st),
                       C.c_uint(pop), C.c_uint(S), C.c_uint(npar)])
        mid = np.asarray(mid, np.float32)
        hoff = np.asarray(hoff, np.float32)
        if model == "oct":
            n_all = len(mid)
            mask = torch.zeros(n_all, dtype=torch.uint8, device="cuda")
            # device copies held in locals: a temporary could be recycled by
            # the allocator for the next one before the launch
            dmid_all, dhoff_all = self._dev(mid), self._dev(hoff)
            self.d.launch(ev["selectTracesForOffsetContinuationTrajectoryAndDifferentialEvolution"],
                          _grid(n_all), THREADS,
                          [self._ptr(dmid_all), self._ptr(dhoff_all), self._ptr(x),
                           C.c_uint(n_all), C.c_uint(S), C.c_uint(pop), C.c_float(dt),
                           C.c_float(apm), C.c_float(m0), C.c_float(h0), self._ptr(mask)])
            sel = np.nonzero(mask.cpu().numpy())[0]
        sel = np.asarray(sel)
        n = int(sel.size)
        smp = self._dev(np.ascontiguousarray(samples[sel], np.float32).ravel() if n
                        else np.zeros(1, np.float32))
        dm = self._dev(mid[sel] if n else np.zeros(1, np.float32))
        dh = self._dev(hoff[sel] if n else np.zeros(1, np.float32))
        dh2 = self._dev((hoff[sel] * hoff[sel]).astype(np.float32) if n
                        else np.zeros(1, np.float32))

        def evaluate(pp, ff):
            if model == "cmp":
                self.d.launch(ev["computeSemblancesForCommonMidPoint"], g, THREADS,
                              [self._ptr(smp), self._ptr(dh2), C.c_uint(n), C.c_uint(S),
                               C.c_uint(pop), C.c_float(dt), C.c_int(tau), C.c_int(w),
                               C.c_uint(ncr), self._ptr(pp), self._ptr(ff)])
            elif model == "zocrs":
                self.d.launch(ev["computeSemblancesForZeroOffsetCommonReflectionSurface"], g,
                              THREADS,
                              [self._ptr(smp), self._ptr(dm), self._ptr(dh2), C.c_uint(n),
                               C.c_uint(S), C.c_uint(pop), C.c_float(m0), C.c_float(dt),
                               C.c_int(tau), C.c_int(w), C.c_uint(ncr), self._ptr(pp),
                               self._ptr(ff)])
            else:
                self.d.launch(ev["computeSemblancesForOffsetContinuationTrajectory"], g, THREADS,
                              [self._ptr(smp), self._ptr(dm), self._ptr(dh), C.c_uint(n),
                               C.c_uint(S), C.c_uint(pop), C.c_float(apm), C.c_float(m0),
                               C.c_float(h0), C.c_float(dt), C.c_int(tau), C.c_int(w),
                               C.c_uint(ncr), self._ptr(nu), self._ptr(pp), self._ptr(ff)])

        # timed from the first evaluation to the best-individual selection
        # (selection and packing excluded, as the engine's kernel_ms)
        e0.record()
        evaluate(x, fx)
        for _ in range(1, gens):
            self.d.launch(ops["mutatePopulations"], g, THREADS,
                          [self._ptr(v), self._ptr(x), self._ptr(dmin), self._ptr(dmax),
                           self._ptr(st), C.c_uint(pop), C.c_uint(S), C.c_uint(npar)])
            self.d.launch(ops["crossoverPopulations"], g, THREADS,
                          [self._ptr(u), self._ptr(x), self._ptr(v), self._ptr(st),
                           C.c_uint(pop), C.c_uint(S), C.c_uint(npar)])
            evaluate(u, fu)
            self.d.launch(ops["nextGeneration"], g, THREADS,
                          [self._ptr(x), self._ptr(fx), self._ptr(u), self._ptr(fu),
                           C.c_uint(pop), C.c_uint(S), C.c_uint(npar), C.c_uint(ncr)])
        best = {"cmp": "selectBestIndividualsForCommonMidPoint",
                "zocrs": "selectBestIndividualsForZeroOffsetCommonReflectionSurface",
                "oct": "selectBestIndividualsForOffsetContinuationTrajectory"}[model]
        self.d.launch(ev[best], _grid(S), THREADS,
                      [self._ptr(x), self._ptr(fx), self._ptr(res), C.c_uint(pop), C.c_uint(S),
                       C.c_uint(ncr)])
        e1.record()
        torch.cuda.synchronize()
        return res.cpu().numpy().reshape(2 + npar, S), e0.elapsed_time(e1), n
