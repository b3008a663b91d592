"""TEST INFRASTRUCTURE: numpy driver of the C lattice oracle (oracle/lbm_oracle.c).

`OracleLBM.step()` performs the reference's CUDA-path step sequence
(fluxcore3D solver/lbm_cuda_ext.py:445-517):
    collide (writes pre-collision macros) -> sponge on f_post -> pull stream
    -> interpolated bounce-back + reset of flow-solid cells (or the in-cell
       swap when there are no links, LBM_CHT.py:1322-1328)
    -> plane boundary conditions in face order (lbm_cuda_ext.py:628-687).
State is the reference's: `f` holds post-stream populations S_k and the macro
arrays hold the macros of S_{k-1}.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

# 8-digit decimal weights of the reference CUDA kernels (solver/lbm_kernels.cu:65-71)
W_CUDA = np.array([0.33333333] + [0.05555556] * 6 + [0.02777778] * 12, dtype=np.float32)
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, -1, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1])
OPP = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15])
FACES = ("+X", "-X", "+Y", "-Y", "+Z", "-Z")


def mrt_matrix() -> np.ndarray:
    """D3Q19 moment basis (d'Humieres et al. 2002) in the reference's row order
    (flow_solver_upgrade.py:98-123), built from the velocity-set polynomials."""
    c2 = CX ** 2 + CY ** 2 + CZ ** 2
    rows = [
        np.ones(19), 19 * c2 - 30, (21 * c2 ** 2 - 53 * c2 + 24) / 2,
        CX, (5 * c2 - 9) * CX, CY, (5 * c2 - 9) * CY, CZ, (5 * c2 - 9) * CZ,
        3 * CX ** 2 - c2, (3 * c2 - 5) * (3 * CX ** 2 - c2),
        CY ** 2 - CZ ** 2, (3 * c2 - 5) * (CY ** 2 - CZ ** 2),
        CX * CY, CY * CZ, CX * CZ,
        (CY ** 2 - CZ ** 2) * CX, (CZ ** 2 - CX ** 2) * CY, (CX ** 2 - CY ** 2) * CZ,
    ]
    return np.array(rows, dtype=np.float64)


def mrt_rates(omega_nu: float, s_e=1.19, s_bulk=1.4, s_ghost=1.2) -> np.ndarray:
    """Relaxation vector of flow_solver_upgrade.py:216-274."""
    S = np.zeros(19)
    S[[9, 11, 13, 14, 15]] = omega_nu
    S[1] = s_e
    S[[2, 4, 6, 8, 10, 12]] = s_bulk
    S[[16, 17, 18]] = s_ghost
    return S


def resolve_face_roles(flow_dir="+X", domain_walls=(), domain_outlets=(), transverse_walls=False) -> dict:
    """pre_post/face_roles.py:3-44."""
    d = flow_dir.upper().strip()
    sign = 1 if d[0] == "+" else -1
    inlet = ("-" if sign > 0 else "+") + d[1]
    outlet = ("+" if sign > 0 else "-") + d[1]
    walls = {s.upper() for s in domain_walls}
    outs = {s.upper() for s in domain_outlets}
    roles = {}
    for f in FACES:
        if f == inlet:
            roles[f] = "inlet"
        elif f in walls:
            roles[f] = "wall"
        elif f == outlet or f in outs:
            roles[f] = "outlet"
        else:
            roles[f] = "wall" if transverse_walls else "periodic"
    return roles


class _Lib:
    _cache: dict = {}

    @classmethod
    def get(cls, real: str):
        if real in cls._cache:
            return cls._cache[real]
        path = build_oracle.lib_path(real)
        if not os.path.exists(path):
            build_oracle.build()
        L = C.CDLL(path)
        vp = C.c_void_p
        i32, i64, f64 = C.c_int, C.c_longlong, C.c_double
        sig = {
            "or_set_constants": [vp, f64, f64],
            "or_macro_collide": [i32, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i64],
            "or_stream_pull": [vp, vp, i32, i32, i32, i32, i32, i32],
            "or_sponge": [vp, vp, vp, vp, vp, vp, i64],
            "or_ibb": [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, i64, i64],
            "or_reset_solid": [vp, vp, i64],
            "or_swap_solid": [vp, vp, i64],
            "or_zou_he": [vp, vp, i32, i32, i32, i32, i32, i32, i32, f64, f64, i32],
            "or_convective": [vp, vp, i32, i32, i32, i32, i32, i32, i32, f64],
        }
        for n, a in sig.items():
            getattr(L, n).argtypes = a
            getattr(L, n).restype = None
        cls._cache[real] = L
        return L


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data


class OracleLBM:
    """Reference CUDA-path lattice solver on the CPU (FP32 or FP64)."""

    def __init__(self, nx, ny, nz, f0, solid_flow, collision="bgk", omega=1.0, omega_minus=None,
                 S=None, Cs_dx2=0.01, sigma=None, links=None, flow_dir="+X", domain_walls=(),
                 domain_outlets=(), transverse_walls=False, u_in_lat=0.05, rho_out_lat=1.0,
                 u_lat_max=0.12, outlet_bc_mode="pressure", real="f32", weights=W_CUDA):
        self.real = real
        self.dt = np.float32 if real == "f32" else np.float64
        self.L = _Lib.get(real)
        w = np.ascontiguousarray(np.asarray(weights, dtype=np.float64))
        self.L.or_set_constants(_p(w), float(np.float32(0.66666667)), float(np.float32(-0.33333333)))
        self.nx, self.ny, self.nz = nx, ny, nz
        self.N = N = nx * ny * nz
        self.f = np.ascontiguousarray(np.asarray(f0, dtype=self.dt).reshape(19, N))
        self.fp = np.empty_like(self.f)
        self.solid = np.ascontiguousarray(np.asarray(solid_flow, dtype=np.uint8).reshape(N))
        self.rho = np.ones(N, self.dt)
        self.u = np.zeros(N, self.dt)
        self.v = np.zeros(N, self.dt)
        self.w = np.zeros(N, self.dt)
        self.mode = {"bgk": 0, "trt": 1, "mrt": 2, "mrt_smag": 3}[collision]
        om = float(omega)
        self.params = np.array([om, om, float(omega_minus or om), float(Cs_dx2), om], dtype=np.float64)
        self.S = np.ascontiguousarray(np.asarray(S if S is not None else np.zeros(19), dtype=np.float64))
        M = mrt_matrix()
        self.M = np.ascontiguousarray(M)
        self.Minv = np.ascontiguousarray(np.linalg.inv(M))
        self.sigma = None if sigma is None else np.ascontiguousarray(np.asarray(sigma, dtype=self.dt).reshape(N))
        self.links = None
        if links is not None and len(links["fluid_flat"]) > 0:
            self.links = {
                "fluid_flat": np.ascontiguousarray(np.asarray(links["fluid_flat"], np.int64)),
                "dir_i": np.ascontiguousarray(np.asarray(links["dir_i"], np.int64)),
                "dir_opp": np.ascontiguousarray(np.asarray(links["dir_opp"], np.int64)),
                "w1": np.ascontiguousarray(np.asarray(links["w_i"], self.dt)),
                "w2": np.ascontiguousarray(np.asarray(links["w_second"], self.dt)),
                "ge": np.ascontiguousarray(np.asarray(links["q_ge_half"], np.uint8)),
                "ff_flat": np.ascontiguousarray(np.asarray(links["ff_flat"], np.int64)),
                "ff_valid": np.ascontiguousarray(np.asarray(links["ff_valid"], np.uint8)),
            }
        roles = resolve_face_roles(flow_dir, domain_walls, domain_outlets, transverse_walls)
        self.periodic = [True, True, True]
        for face, r in roles.items():
            if r in ("inlet", "outlet", "wall"):
                self.periodic["XYZ".index(face[1])] = False
        d = flow_dir.upper().strip()
        fsg = 1 if d[0] == "+" else -1
        fax = "XYZ".index(d[1])
        u_signed = float(max(-u_lat_max, min(u_lat_max, u_in_lat * fsg)))
        self.bcs = []
        for face, r in roles.items():
            if r not in ("inlet", "outlet"):
                continue
            ax = "XYZ".index(face[1])
            n = (nx, ny, nz)[ax]
            pidx, sgn = (n - 1, 1) if face[0] == "+" else (0, -1)
            iidx = pidx - 1 if pidx > 0 else 1
            if r == "inlet":
                self.bcs.append(("zh", ax, pidx, iidx, 0, u_signed, rho_out_lat, fsg))
            elif outlet_bc_mode == "convective" and ax == fax:
                self.bcs.append(("cv", ax, pidx, iidx, 1 if pidx == 0 else -1, u_signed, rho_out_lat, sgn))
            else:
                self.bcs.append(("zh", ax, pidx, iidx, 1, u_signed, rho_out_lat, sgn))

    def collide(self):
        self.L.or_macro_collide(self.mode, _p(self.f), _p(self.fp), _p(self.rho), _p(self.u), _p(self.v),
                                _p(self.w), _p(self.solid), _p(self.params), _p(self.S), _p(self.M),
                                _p(self.Minv), self.N)

    def step(self, n: int = 1):
        L = self.L
        for _ in range(n):
            self.collide()
            if self.sigma is not None:
                L.or_sponge(_p(self.fp), _p(self.rho), _p(self.u), _p(self.v), _p(self.w), _p(self.sigma), self.N)
            L.or_stream_pull(_p(self.fp), _p(self.f), self.nx, self.ny, self.nz, *[int(p) for p in self.periodic])
            if self.links is not None:
                k = self.links
                L.or_ibb(_p(self.fp), _p(self.f), _p(k["fluid_flat"]), _p(k["dir_i"]), _p(k["dir_opp"]),
                         _p(k["w1"]), _p(k["w2"]), _p(k["ge"]), _p(k["ff_flat"]), _p(k["ff_valid"]),
                         len(k["fluid_flat"]), self.N)
                L.or_reset_solid(_p(self.f), _p(self.solid), self.N)
            else:
                L.or_swap_solid(_p(self.f), _p(self.solid), self.N)
            for kind, ax, pidx, iidx, code, us, ro, sg in self.bcs:
                if kind == "zh":
                    L.or_zou_he(_p(self.f), _p(self.solid), self.nx, self.ny, self.nz, ax, pidx, iidx, code,
                                us, ro, sg)
                else:
                    L.or_convective(_p(self.f), _p(self.solid), self.nx, self.ny, self.nz, ax, pidx, iidx,
                                    code, ro)
