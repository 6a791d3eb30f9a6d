"""numpy interpreter of libtdcc program op lists (from tdcc_program_json).

Executes exactly the GEMM mode groups / strides / coefficients and the
elementwise terms the GPU kernels receive, on flat host buffers, so the
equation programs and their prologue/stage split can be checked on a CPU."""
import numpy as np

S_TEI, S_F, S_T1, S_T2, S_L1, S_L2, S_OUT, S_MU, S_RES = range(9)


def _group(g):
    n = g["n"]
    if n == 0:
        z = np.zeros(1, dtype=np.int64)
        return z, z
    idx = np.indices(g["dim"]).reshape(n, -1).astype(np.int64)
    s0 = np.array(g["s0"], dtype=np.int64)[:, None]
    s1 = np.array(g["s1"], dtype=np.int64)[:, None]
    return (idx * s0).sum(0), (idx * s1).sum(0)


class Emulator:
    """``share``: workspace slots the program maps to one buffer ("buf") alias
    the same memory, as on the device (off for reverse-mode checks, which
    read every forward value after the forward ran -- the runtime turns the
    sharing off for them too)."""

    def __init__(self, prog, o, v, n_mu=3, share=True, zero=False):
        self.p = prog
        self.o, self.v, self.n = o, v, o + v
        self.n_mu = n_mu
        self.bufs = {}
        groups = {}
        for i, s in enumerate(prog["slots"]):
            if s["fixed"]:
                continue
            b = s.get("buf", i) if share else i
            size = {0: 8, 1: 16, 2: 1}[s["dt"]] * s["numel"]
            groups.setdefault(b, []).append((i, s, size))
        for b, members in groups.items():
            # workspace starts as NaN (all-ones bytes): an op that reads what no op wrote shows
            # up; reverse-mode programs accumulate, their workspace starts at zero (zero=True),
            # as the runtime allocates it
            raw = bytearray((b"\x00" if zero else b"\xff") * max(sz for _, _, sz in members))
            for i, s, _ in members:
                dt = {0: np.float64, 1: np.complex128, 2: np.uint8}[s["dt"]]
                arr = np.frombuffer(raw, dtype=dt, count=s["numel"])
                if s["ones"]:
                    arr[:] = 1
                self.bufs[i] = arr

    def bind(self, slot, arr):
        self.bufs[slot] = np.ascontiguousarray(arr).reshape(-1)

    def run(self, phase="all"):
        for op in self.p["ops"]:
            if phase == "setup" and not op.get("const"):
                continue
            if phase == "prologue" and (op["varying"] or op.get("const")):
                continue
            if phase == "stage" and not op["varying"]:
                continue
            getattr(self, "_" + op["kind"])(op)

    def _gemm(self, op):
        am, cm = _group(op["gm"])
        bn, cn = _group(op["gn"])
        ak, bk = _group(op["gk"])
        A = self.bufs[op["sa"]]
        B = self.bufs[op["sb"]]
        C = self.bufs[op["sc"]]
        for z in range(op.get("nb", 1)):
            Am = A[op["oa"] + z * op.get("bsA", 0) + am[:, None] + ak[None, :]]
            Bm = B[op["ob"] + z * op.get("bsB", 0) + bk[:, None] + bn[None, :]]
            val = complex(op["ar"], op["ai"]) * (Am @ Bm)
            if C.dtype == np.float64:
                val = val.real
            idx = op["oc"] + z * op.get("bsC", 0) + cm[:, None] + cn[None, :]
            if op["acc"] or op["atomic"]:
                C[idx] += val
            else:
                C[idx] = val

    def _add(self, op):
        d = op["d"]
        I = np.indices(d).reshape(len(d), -1).astype(np.int64)
        C = self.bufs[op["sc"]]
        offc = op["oc"] + (I * np.array(op["sC"], dtype=np.int64)[:, None]).sum(0)
        s = np.zeros(I.shape[1], dtype=np.complex128)
        for t in op["terms"]:
            A = self.bufs[t["sa"]]
            x = A[t["oa"] + (I * np.array(t["sA"], dtype=np.int64)[:, None]).sum(0)].astype(np.complex128)
            if t["sb"] >= 0:
                B = self.bufs[t["sb"]]
                x = x * B[t["ob"] + (I * np.array(t["sB"], dtype=np.int64)[:, None]).sum(0)]
            s += complex(t["cr"], t["ci"]) * x
        if C.dtype == np.float64:
            s = s.real
        if op["acc"]:
            C[offc] += s
        else:
            C[offc] = s

    def _reduce(self, op):
        out = self.bufs[op["out"]]
        X = self.bufs[op["x"]]
        Y = self.bufs[op["y"]] if op["y"] >= 0 else None
        do, dr = op["dout"], op["dred"]
        Io = np.indices(do).reshape(len(do), -1).astype(np.int64) if do else np.zeros((0, 1), np.int64)
        Ir = np.indices(dr).reshape(len(dr), -1).astype(np.int64) if dr else np.zeros((0, 1), np.int64)
        def off(I, s):
            return (I * np.array(s, dtype=np.int64)[:, None]).sum(0) if len(s) else np.zeros(I.shape[1], np.int64)
        xo = op["ox"] + off(Io, op["so_x"])[:, None] + off(Ir, op["sr_x"])[None, :]
        v = X[xo].astype(np.complex128)
        if Y is not None:
            yo = op["oy"] + off(Io, op["so_y"])[:, None] + off(Ir, op["sr_y"])[None, :]
            v = v * Y[yo]
        r = complex(op["cr"], op["ci"]) * v.sum(1)
        oo = op["oout"] + off(Io, op["so_out"])
        if op["acc"]:
            out[oo] += r
        else:
            out[oo] = r

    def _trace(self, op):
        o, v, n = self.o, self.v, self.n
        dij, l1, dai, dab = (self.bufs[k] for k in op["slots"])
        mu = self.bufs[S_MU]
        res = self.bufs[S_RES]
        bs = op.get("bs", [0, 0, 0, 0])
        for z in range(op.get("nb", 1)):
            rho = np.zeros((n, n), dtype=np.complex128)
            rho[:o, :o] = dij[z * bs[0]:][: o * o].reshape(o, o)
            rho[:o, o:] = l1[z * bs[1]:][: o * v].reshape(o, v)
            rho[o:, :o] = dai[z * bs[2]:][: v * o].reshape(v, o)
            rho[o:, o:] = dab[z * bs[3]:][: v * v].reshape(v, v)
            for k in range(op["n_mu"]):
                res[z * op.get("bsres", 0) + k] = (mu[k * n * n:(k + 1) * n * n].reshape(n, n) * rho).sum()
