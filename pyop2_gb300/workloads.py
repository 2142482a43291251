"""Local kernels and problem builders of the benchmark configurations.

The kernels are ordinary PyOP2 C kernels (strings), as a user would write
them; the builders take the ``op2`` module to use, so the same problem can be
set up on pyop2_gb300 and on any other implementation of the PyOP2 API.

Hand counts of FP64 operations per cell (FMA = 2) are given with each kernel;
they are the algorithmic flops of the roofline.
"""
import numpy as np

from pyop2_gb300 import meshes

# ---------------------------------------------------------------- 2D P1
# y_e += K_e x_e with the 3x3 P1 stiffness matrix formed explicitly, plus the
# cell area summed into a Global.  ~60 flops/cell.
P1_2D_LAPLACE = r"""
static void p1_laplace_2d(double *y, const double *restrict X, const double *restrict x,
                          double *area)
{
  const double j00 = X[2] - X[0], j01 = X[4] - X[0];
  const double j10 = X[3] - X[1], j11 = X[5] - X[1];
  const double det = j00 * j11 - j01 * j10;
  const double a = 0.5 * fabs(det);
  /* gradients of the three hat functions: rows of J^{-T} applied to the
     reference gradients (-1,-1), (1,0), (0,1) */
  const double id = 1.0 / det;
  double g[3][2];
  g[1][0] =  j11 * id; g[1][1] = -j01 * id;
  g[2][0] = -j10 * id; g[2][1] =  j00 * id;
  g[0][0] = -g[1][0] - g[2][0]; g[0][1] = -g[1][1] - g[2][1];
  double K[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      K[i][j] = a * (g[i][0] * g[j][0] + g[i][1] * g[j][1]);
  for (int i = 0; i < 3; ++i)
    y[i] += K[i][0] * x[0] + K[i][1] * x[1] + K[i][2] * x[2];
  area[0] += a;
}
"""
P1_2D_FLOPS = 60

# ---------------------------------------------------------------- 3D P1
# Matrix-free P1 tetrahedral Laplacian action: y_e += vol * G G^T x_e written
# as w = C^T (C d) / (6 |det J|), C the cofactor matrix of J, d = x_k - x_0.
# Flops: J 9, cofactors 27, det 5, d 3, C d 15, C^T(.) 15, scale 1 div + 4,
# y0 3  -> ~82 + one division.
P1_3D_LAPLACE_ACTION = r"""
static void p1_laplace_3d(double *restrict y, const double *restrict X,
                          const double *restrict x)
{
  const double a0 = X[3] - X[0], a1 = X[4] - X[1], a2 = X[5]  - X[2];
  const double b0 = X[6] - X[0], b1 = X[7] - X[1], b2 = X[8]  - X[2];
  const double c0 = X[9] - X[0], c1 = X[10] - X[1], c2 = X[11] - X[2];
  /* J has columns a, b, c; C = cofactor matrix of J (J^{-T} = C / det) */
  const double C00 = b1 * c2 - b2 * c1, C01 = b2 * c0 - b0 * c2, C02 = b0 * c1 - b1 * c0;
  const double C10 = a2 * c1 - a1 * c2, C11 = a0 * c2 - a2 * c0, C12 = a1 * c0 - a0 * c1;
  const double C20 = a1 * b2 - a2 * b1, C21 = a2 * b0 - a0 * b2, C22 = a0 * b1 - a1 * b0;
  const double det = a0 * C00 + a1 * C01 + a2 * C02;
  const double d0 = x[1] - x[0], d1 = x[2] - x[0], d2 = x[3] - x[0];
  /* J^{-T} d scaled by det: rows of C are the cofactors of J's columns */
  const double v0 = C00 * d0 + C10 * d1 + C20 * d2;
  const double v1 = C01 * d0 + C11 * d1 + C21 * d2;
  const double v2 = C02 * d0 + C12 * d1 + C22 * d2;
  const double s = 1.0 / (6.0 * fabs(det));
  const double w1 = (C00 * v0 + C01 * v1 + C02 * v2) * s;
  const double w2 = (C10 * v0 + C11 * v1 + C12 * v2) * s;
  const double w3 = (C20 * v0 + C21 * v1 + C22 * v2) * s;
  y[0] -= w1 + w2 + w3;
  y[1] += w1;
  y[2] += w2;
  y[3] += w3;
}
"""
P1_3D_FLOPS = 84
P1_3D_BYTES_PER_CELL = None  # computed by bytes_c2a()

# 4x4 element stiffness matrix into a Mat (assembly of the same operator).
P1_3D_LAPLACE_MATRIX = r"""
static void p1_laplace_3d_mat(double A[4][4], const double *restrict X)
{
  const double a0 = X[3] - X[0], a1 = X[4] - X[1], a2 = X[5]  - X[2];
  const double b0 = X[6] - X[0], b1 = X[7] - X[1], b2 = X[8]  - X[2];
  const double c0 = X[9] - X[0], c1 = X[10] - X[1], c2 = X[11] - X[2];
  const double C00 = b1 * c2 - b2 * c1, C01 = b2 * c0 - b0 * c2, C02 = b0 * c1 - b1 * c0;
  const double C10 = a2 * c1 - a1 * c2, C11 = a0 * c2 - a2 * c0, C12 = a1 * c0 - a0 * c1;
  const double C20 = a1 * b2 - a2 * b1, C21 = a2 * b0 - a0 * b2, C22 = a0 * b1 - a1 * b0;
  const double det = a0 * C00 + a1 * C01 + a2 * C02;
  const double s = 1.0 / (6.0 * fabs(det));
  /* gradients times det: g_1..3 = rows of C^T ... columns: g_k = (C0k-1...) */
  double g[4][3];
  g[1][0] = C00; g[1][1] = C01; g[1][2] = C02;
  g[2][0] = C10; g[2][1] = C11; g[2][2] = C12;
  g[3][0] = C20; g[3][1] = C21; g[3][2] = C22;
  for (int k = 0; k < 3; ++k) g[0][k] = -g[1][k] - g[2][k] - g[3][k];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      A[i][j] += s * (g[i][0] * g[j][0] + g[i][1] * g[j][1] + g[i][2] * g[j][2]);
}
"""
P1_3D_MATRIX_FLOPS = 120


def bytes_c2a(ncells, nverts):
    """Compulsory bytes of one y += K x action: map read once, coords and x
    read once, y read and written once."""
    return ncells * 4 * 4 + nverts * (3 * 8 + 8 + 2 * 8)


def build_p1_2d(op2, n=64, seed=0):
    """Config 1: 2D P1 Laplacian action + area Global on an n x n split square."""
    coords, cells = meshes.unit_square_tris(n, jitter=0.2, seed=seed)
    rng = np.random.default_rng(seed + 1)
    V, C = coords.shape[0], cells.shape[0]
    verts = op2.Set(V, "vertices")
    cset = op2.Set(C, "cells")
    c2v = op2.Map(cset, verts, 3, cells, "cell2vert")
    X = op2.Dat(verts ** 2, coords, np.float64, "coords")
    x = op2.Dat(verts, rng.uniform(-1, 1, V), np.float64, "x")
    y = op2.Dat(verts, np.zeros(V), np.float64, "y")
    area = op2.Global(1, 0.0, np.float64, "area")
    k = op2.Kernel(P1_2D_LAPLACE, "p1_laplace_2d")

    def run():
        op2.par_loop(k, cset, y(op2.INC, c2v), X(op2.READ, c2v), x(op2.READ, c2v),
                     area(op2.INC))
    return dict(run=run, y=y, area=area, cells=cset, verts=verts, c2v=c2v, X=X, x=x, kernel=k)


def build_p1_3d(op2, n=128, permute=False, seed=0):
    """Config 2a: matrix-free P1 tetrahedral Laplacian action on n^3 x 6 tets."""
    coords, cells = meshes.unit_cube_tets(n, permute=permute, seed=seed)
    rng = np.random.default_rng(seed + 1)
    V, C = coords.shape[0], cells.shape[0]
    verts = op2.Set(V, "vertices")
    cset = op2.Set(C, "cells")
    c2v = op2.Map(cset, verts, 4, cells, "cell2vert")
    X = op2.Dat(verts ** 3, coords, np.float64, "coords")
    x = op2.Dat(verts, rng.uniform(-1, 1, V), np.float64, "x")
    y = op2.Dat(verts, np.zeros(V), np.float64, "y")
    k = op2.Kernel(P1_3D_LAPLACE_ACTION, "p1_laplace_3d")

    def run():
        op2.par_loop(k, cset, y(op2.INC, c2v), X(op2.READ, c2v), x(op2.READ, c2v))
    return dict(run=run, y=y, cells=cset, verts=verts, c2v=c2v, X=X, x=x, kernel=k,
                coords=coords, cellmap=cells)


# ------------------------------------------------------- nonlinear residual
# F(u)_i = sum_e int kappa_e (1 + u^2) grad u . grad v_i - f v_i, P1 tets, f = 1.
# With C the cofactor matrix (rows b x c, c x a, a x b) and d = u_k - u_0:
#   v = C^T d = det grad u,  G_0 = -(C_0 + C_1 + C_2), G_k = C_{k-1},
#   q = (sum u_i^2 + (sum u_i)^2) / 20 = (1/vol) int u^2,
#   F_i = kappa (1 + q) (G_i . v) / (6 |det|) - |det| / 24.
_TET_GEOM = r"""
  const double a0 = X[3] - X[0], a1 = X[4] - X[1], a2 = X[5]  - X[2];
  const double b0 = X[6] - X[0], b1 = X[7] - X[1], b2 = X[8]  - X[2];
  const double c0 = X[9] - X[0], c1 = X[10] - X[1], c2 = X[11] - X[2];
  const double C00 = b1 * c2 - b2 * c1, C01 = b2 * c0 - b0 * c2, C02 = b0 * c1 - b1 * c0;
  const double C10 = a2 * c1 - a1 * c2, C11 = a0 * c2 - a2 * c0, C12 = a1 * c0 - a0 * c1;
  const double C20 = a1 * b2 - a2 * b1, C21 = a2 * b0 - a0 * b2, C22 = a0 * b1 - a1 * b0;
  const double det = a0 * C00 + a1 * C01 + a2 * C02;
  const double adet = fabs(det);
  const double s = 1.0 / (6.0 * adet);
  const double d0 = u[1] - u[0], d1 = u[2] - u[0], d2 = u[3] - u[0];
  const double v0 = C00 * d0 + C10 * d1 + C20 * d2;
  const double v1 = C01 * d0 + C11 * d1 + C21 * d2;
  const double v2 = C02 * d0 + C12 * d1 + C22 * d2;
  const double S = u[0] + u[1] + u[2] + u[3];
  const double q = (u[0] * u[0] + u[1] * u[1] + u[2] * u[2] + u[3] * u[3] + S * S) * 0.05;
"""

NL_RESIDUAL = r"""
static void nl_residual(double *restrict F, const double *restrict X,
                        const double *restrict u, const double *restrict kappa)
{""" + _TET_GEOM + r"""
  const double c = kappa[0] * (1.0 + q) * s;
  const double f4 = adet * (1.0 / 24.0);
  const double w1 = c * (C00 * v0 + C01 * v1 + C02 * v2);
  const double w2 = c * (C10 * v0 + C11 * v1 + C12 * v2);
  const double w3 = c * (C20 * v0 + C21 * v1 + C22 * v2);
  F[0] += -(w1 + w2 + w3) - f4;
  F[1] += w1 - f4;
  F[2] += w2 - f4;
  F[3] += w3 - f4;
}
"""
NL_RESIDUAL_FLOPS = 120

# Vector-Jacobian product: given lambda on the vertices, L = lambda . F;
#   vl = C^T (lambda_k - lambda_0),  gg = vl . v,
#   dL/dkappa_e = (1 + q) gg / (6 |det|),
#   dL/du_j += kappa / (6|det|) [ (u_j + S)/10 gg + (1 + q) (G_j . vl) ].
NL_RESIDUAL_VJP = r"""
static void nl_residual_vjp(const double *restrict lam, const double *restrict X,
                            const double *restrict u, const double *restrict kappa,
                            double *restrict du, double *restrict dkappa)
{""" + _TET_GEOM + r"""
  const double l0 = lam[1] - lam[0], l1 = lam[2] - lam[0], l2 = lam[3] - lam[0];
  const double vl0 = C00 * l0 + C10 * l1 + C20 * l2;
  const double vl1 = C01 * l0 + C11 * l1 + C21 * l2;
  const double vl2 = C02 * l0 + C12 * l1 + C22 * l2;
  const double gg = vl0 * v0 + vl1 * v1 + vl2 * v2;
  const double b = 1.0 + q;
  dkappa[0] = b * gg * s;
  const double a = kappa[0] * s;
  const double t1 = C00 * vl0 + C01 * vl1 + C02 * vl2;
  const double t2 = C10 * vl0 + C11 * vl1 + C12 * vl2;
  const double t3 = C20 * vl0 + C21 * vl1 + C22 * vl2;
  const double h = 0.1 * gg;
  du[0] += a * ((u[0] + S) * h - b * (t1 + t2 + t3));
  du[1] += a * ((u[1] + S) * h + b * t1);
  du[2] += a * ((u[2] + S) * h + b * t2);
  du[3] += a * ((u[3] + S) * h + b * t3);
}
"""
NL_RESIDUAL_VJP_FLOPS = 170

# Forward and VJP in one pass (lambda known when the residual is evaluated):
# the geometry and grad u are computed once.
NL_RESIDUAL_FUSED = r"""
static void nl_residual_fused(double *restrict F, const double *restrict lam,
                              const double *restrict X, const double *restrict u,
                              const double *restrict kappa, double *restrict du,
                              double *restrict dkappa)
{""" + _TET_GEOM + r"""
  const double b = 1.0 + q;
  const double a = kappa[0] * s;
  const double c = a * b;
  const double f4 = adet * (1.0 / 24.0);
  const double w1 = C00 * v0 + C01 * v1 + C02 * v2;
  const double w2 = C10 * v0 + C11 * v1 + C12 * v2;
  const double w3 = C20 * v0 + C21 * v1 + C22 * v2;
  F[0] += -c * (w1 + w2 + w3) - f4;
  F[1] += c * w1 - f4;
  F[2] += c * w2 - f4;
  F[3] += c * w3 - f4;
  const double l0 = lam[1] - lam[0], l1 = lam[2] - lam[0], l2 = lam[3] - lam[0];
  /* gg = vl . v = (lam - lam_0) . (w1, w2, w3) since w_k = C_k . v */
  const double gg = l0 * w1 + l1 * w2 + l2 * w3;
  const double vl0 = C00 * l0 + C10 * l1 + C20 * l2;
  const double vl1 = C01 * l0 + C11 * l1 + C21 * l2;
  const double vl2 = C02 * l0 + C12 * l1 + C22 * l2;
  dkappa[0] = b * gg * s;
  const double t1 = C00 * vl0 + C01 * vl1 + C02 * vl2;
  const double t2 = C10 * vl0 + C11 * vl1 + C12 * vl2;
  const double t3 = C20 * vl0 + C21 * vl1 + C22 * vl2;
  const double h = 0.1 * gg;
  du[0] += a * ((u[0] + S) * h - b * (t1 + t2 + t3));
  du[1] += a * ((u[1] + S) * h + b * t1);
  du[2] += a * ((u[2] + S) * h + b * t2);
  du[3] += a * ((u[3] + S) * h + b * t3);
}
"""

# Jacobian dF/du as 4x4 element blocks (for J^T lambda checks):
#   J_ij = kappa / (6|det|) [ (u_j + S)/10 (G_i . v) + (1 + q) (G_i . G_j) ].
NL_RESIDUAL_JACOBIAN = r"""
static void nl_residual_jac(double A[4][4], const double *restrict X,
                            const double *restrict u, const double *restrict kappa)
{""" + _TET_GEOM + r"""
  double G[4][3] = {{0, 0, 0}, {C00, C01, C02}, {C10, C11, C12}, {C20, C21, C22}};
  for (int k = 0; k < 3; ++k) G[0][k] = -(G[1][k] + G[2][k] + G[3][k]);
  const double a = kappa[0] * s, b = 1.0 + q;
  for (int i = 0; i < 4; ++i) {
    const double gv = G[i][0] * v0 + G[i][1] * v1 + G[i][2] * v2;
    for (int j = 0; j < 4; ++j)
      A[i][j] += a * ((u[j] + S) * 0.1 * gv +
                      b * (G[i][0] * G[j][0] + G[i][1] * G[j][1] + G[i][2] * G[j][2]));
  }
}
"""


def build_nonlinear(op2, n=64, seed=0):
    """Config 4 data: P1 tets of an n^3 cube, u ~ U[-1,1], kappa ~ lognormal(0, 0.5)
    per cell, lambda ~ U[-1,1] (seeded)."""
    coords, cells = meshes.unit_cube_tets(n, permute=False, seed=seed)
    rng = np.random.default_rng(seed + 7)
    V, C = coords.shape[0], cells.shape[0]
    verts = op2.Set(V, "vertices")
    cset = op2.Set(C, "cells")
    c2v = op2.Map(cset, verts, 4, cells, "cell2vert")
    X = op2.Dat(verts ** 3, coords, np.float64, "coords")
    u = rng.uniform(-1, 1, V)
    kappa = rng.lognormal(0.0, 0.5, C)
    lam = rng.uniform(-1, 1, V)
    return dict(verts=verts, cells=cset, c2v=c2v, X=X, u=u, kappa=kappa, lam=lam,
                coords=coords, cellmap=cells)


# ------------------------------------------------------------ P2 triangles
def _p2_reference_matrices():
    """Exact reference-triangle integrals of the P2 basis (v0, v1, v2, e12,
    e02, e01): mass M and stiffness blocks K_ab = int d_a phi_i d_b phi_j.
    Monomials integrate exactly: int_T xi^a eta^b = a! b! / (a + b + 2)!."""
    from math import factorial
    # polynomials as {(a, b): coeff} in xi, eta
    L = [{(0, 0): 1.0, (1, 0): -1.0, (0, 1): -1.0}, {(1, 0): 1.0}, {(0, 1): 1.0}]

    def mul(p, q):
        r = {}
        for (a, b), c in p.items():
            for (d, e), f in q.items():
                r[(a + d, b + e)] = r.get((a + d, b + e), 0.0) + c * f
        return r

    def add(p, q, s=1.0):
        r = dict(p)
        for k, v in q.items():
            r[k] = r.get(k, 0.0) + s * v
        return r

    def scale(p, s):
        return {k: s * v for k, v in p.items()}

    def deriv(p, axis):
        r = {}
        for (a, b), c in p.items():
            if axis == 0 and a > 0:
                r[(a - 1, b)] = r.get((a - 1, b), 0.0) + a * c
            if axis == 1 and b > 0:
                r[(a, b - 1)] = r.get((a, b - 1), 0.0) + b * c
        return r

    def integ(p):
        return sum(c * factorial(a) * factorial(b) / factorial(a + b + 2) for (a, b), c in p.items())

    phi = [add(scale(mul(L[i], L[i]), 2.0), L[i], -1.0) for i in range(3)]
    phi += [scale(mul(L[1], L[2]), 4.0), scale(mul(L[0], L[2]), 4.0), scale(mul(L[0], L[1]), 4.0)]
    M = np.array([[integ(mul(a, b)) for b in phi] for a in phi])
    K = {}
    for ax in range(2):
        for bx in range(2):
            K[(ax, bx)] = np.array([[integ(mul(deriv(a, ax), deriv(b, bx))) for b in phi]
                                    for a in phi])
    return M, K


def _p2_kernel():
    M, K = _p2_reference_matrices()
    mats = [M, K[(0, 0)], K[(0, 1)] + K[(1, 0)], K[(1, 1)]]
    lines = [r"""static void p2_mass_laplace(double *restrict y, const double *restrict X,
                            const double *restrict x, double *restrict norm)
{
  const double j00 = X[2] - X[0], j01 = X[4] - X[0];
  const double j10 = X[3] - X[1], j11 = X[5] - X[1];
  const double det = j00 * j11 - j01 * j10;
  const double adet = fabs(det), ia = 1.0 / adet;
  /* G = |det| J^{-1} J^{-T} */
  const double G00 = (j11 * j11 + j01 * j01) * ia;
  const double G01 = -(j10 * j11 + j00 * j01) * ia;
  const double G11 = (j10 * j10 + j00 * j00) * ia;
  const double w[4] = {adet, G00, G01, G11};"""]
    flops = 20
    for i in range(6):
        terms = []
        for m, R in enumerate(mats):
            row = " + ".join("%.17g * x[%d]" % (R[i, j], j) for j in range(6) if R[i, j] != 0.0)
            if row:
                terms.append("w[%d] * (%s)" % (m, row))
                flops += 2 * sum(1 for j in range(6) if R[i, j] != 0.0) + 2
        lines.append("  const double c%d = %s;" % (i, " + ".join(terms)))
    for i in range(6):
        lines.append("  y[%d] += c%d;" % (i, i))
    lines.append("  norm[0] += c0 * c0 + c1 * c1 + c2 * c2 + c3 * c3 + c4 * c4 + c5 * c5;")
    lines.append("}")
    flops += 12
    return "\n".join(lines) + "\n", flops


P2_MASS_LAPLACE, P2_FLOPS = _p2_kernel()


def build_p2_batch(op2, sizes, seed=0):
    """Config 3: one P2 mass+Laplace action problem per grid size n in sizes."""
    out = []
    k = op2.Kernel(P2_MASS_LAPLACE, "p2_mass_laplace")
    for i, n in enumerate(sizes):
        coords, cells, c2d, ndofs = meshes.p2_square(n, jitter=0.2, seed=seed + i)
        rng = np.random.default_rng(seed + 1000 + i)
        verts = op2.Set(coords.shape[0])
        dofs = op2.Set(ndofs)
        cset = op2.Set(cells.shape[0])
        c2v = op2.Map(cset, verts, 3, cells)
        cmap = op2.Map(cset, dofs, 6, c2d)
        X = op2.Dat(verts ** 2, coords, np.float64)
        x = op2.Dat(dofs, rng.uniform(-1, 1, ndofs), np.float64)
        y = op2.Dat(dofs, np.zeros(ndofs), np.float64)
        g = op2.Global(1, 0.0, np.float64)
        out.append(dict(cells=cset, c2v=c2v, c2d=cmap, X=X, x=x, y=y, g=g, kernel=k,
                        args=(y(op2.INC, cmap), X(op2.READ, c2v), x(op2.READ, cmap),
                              g(op2.INC))))
    return out


# ---------------------------------------------------- extruded P1 prisms
# Linear elasticity sigma = lambda tr(grad u) I + mu (grad u + grad u^T) on
# straight vertical prisms: node (a, k) = base vertex a (0..2), level k (0
# bottom, 1 top); N_ak = lambda_a(xi, eta) phi_k(zeta).  The in-plane
# gradients of lambda_a are constant, d/dz N_ak = lambda_a phi_k' / h.
# Quadrature: 3-point degree-2 triangle rule x 2-point Gauss in zeta, exact
# for the integrands (degree 2 in (xi, eta) and in zeta).  Dats of the
# displacement have shape (NRHS, 3) per node, packed [node][rhs][component].
PRISM_NRHS = 8

_PRISM_GEOM = r"""
  const double j00 = X[3] - X[0], j01 = X[6] - X[0];
  const double j10 = X[4] - X[1], j11 = X[7] - X[1];
  const double det2 = j00 * j11 - j01 * j10;
  const double h = X[11] - X[2];
  const double id = 1.0 / det2;
  double g[3][2];
  g[1][0] = j11 * id;  g[1][1] = -j01 * id;
  g[2][0] = -j10 * id; g[2][1] = j00 * id;
  g[0][0] = -g[1][0] - g[2][0]; g[0][1] = -g[1][1] - g[2][1];
  const double ih = 1.0 / h;
  const double vol = fabs(det2 * h);
  const double wq = vol * (1.0 / 12.0);   /* 6 points: 1/6 (triangle) x 1/2 (Gauss) */
  const double TL[3][3] = {{2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0},
                           {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0},
                           {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0}};
  const double ZQ[2] = {0.5 - 0.28867513459481287, 0.5 + 0.28867513459481287};
"""

# grad of field F (indexed F[(node * NRHS + r) * 3 + c]) at quadrature point
# (tq, zq) into du[c][d]; Gx/Gy/D precomputed per rhs.
_PRISM_PREP = r"""
    double Gx[2][3], Gy[2][3], D[3][3];
    for (int c = 0; c < 3; ++c) {
      for (int k = 0; k < 2; ++k) {
        double sx = 0.0, sy = 0.0;
        for (int a = 0; a < 3; ++a) {
          const double v = FIELD[((a + 3 * k) * NRHS + r) * 3 + c];
          sx += g[a][0] * v; sy += g[a][1] * v;
        }
        Gx[k][c] = sx; Gy[k][c] = sy;
      }
      for (int a = 0; a < 3; ++a)
        D[a][c] = (FIELD[((a + 3) * NRHS + r) * 3 + c] - FIELD[(a * NRHS + r) * 3 + c]) * ih;
    }
"""


def _prism_prep(field, prefix):
    return (_PRISM_PREP.replace("FIELD", field).replace("Gx", prefix + "Gx")
            .replace("Gy", prefix + "Gy").replace("D[", prefix + "D["))


_PRISM_GRAD = r"""
        double PRE_du[3][3];
        for (int c = 0; c < 3; ++c) {
          PRE_du[c][0] = z0 * PRE_Gx[0][c] + z1 * PRE_Gx[1][c];
          PRE_du[c][1] = z0 * PRE_Gy[0][c] + z1 * PRE_Gy[1][c];
          PRE_du[c][2] = TL[tq][0] * PRE_D[0][c] + TL[tq][1] * PRE_D[1][c] + TL[tq][2] * PRE_D[2][c];
        }
"""


def _prism_grad(prefix):
    return _PRISM_GRAD.replace("PRE_", prefix)


PRISM_ELASTICITY_ACTION = (r"""
#define NRHS %d
static void prism_elasticity(double *restrict y, const double *restrict X,
                             const double *restrict u, const double *restrict lame)
{""" % PRISM_NRHS + _PRISM_GEOM + r"""
  const double lam = lame[0], mu = lame[1];
  for (int r = 0; r < NRHS; ++r) {""" + _prism_prep("u", "u") + r"""
    double Sxy[2][3][2] = {{{0}}}, T[3][3] = {{0}};
    for (int zq = 0; zq < 2; ++zq) {
      const double z1 = ZQ[zq], z0 = 1.0 - z1;
      for (int tq = 0; tq < 3; ++tq) {""" + _prism_grad("u") + r"""
        const double tr = udu[0][0] + udu[1][1] + udu[2][2];
        double s[3][3];
        for (int c = 0; c < 3; ++c)
          for (int d = 0; d < 3; ++d)
            s[c][d] = mu * (udu[c][d] + udu[d][c]) + (c == d ? lam * tr : 0.0);
        const double w0 = wq * z0, w1 = wq * z1;
        for (int c = 0; c < 3; ++c) {
          Sxy[0][c][0] += w0 * s[c][0]; Sxy[0][c][1] += w0 * s[c][1];
          Sxy[1][c][0] += w1 * s[c][0]; Sxy[1][c][1] += w1 * s[c][1];
          for (int a = 0; a < 3; ++a) T[a][c] += wq * TL[tq][a] * s[c][2];
        }
      }
    }
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) {
        const double xy0 = g[a][0] * Sxy[0][c][0] + g[a][1] * Sxy[0][c][1];
        const double xy1 = g[a][0] * Sxy[1][c][0] + g[a][1] * Sxy[1][c][1];
        y[(a * NRHS + r) * 3 + c] += xy0 - T[a][c] * ih;
        y[((a + 3) * NRHS + r) * 3 + c] += xy1 + T[a][c] * ih;
      }
  }
}
#undef NRHS
""").replace("udu", "udu")
PRISM_ACTION_FLOPS_PER_RHS = 800

# Adjoint of L = sum_r w_r . y_r with y_r = K(lambda, mu) u_r:
#   dL/du_r = K w_r (K symmetric), dL/dlambda = sum_r int tr(grad w_r) tr(grad u_r),
#   dL/dmu = sum_r int 2 eps(w_r) : eps(u_r).
PRISM_ELASTICITY_VJP = (r"""
#define NRHS %d
static void prism_elasticity_vjp(const double *restrict w, const double *restrict X,
                                 const double *restrict u, const double *restrict lame,
                                 double *restrict du, double *restrict dlame)
{""" % PRISM_NRHS + _PRISM_GEOM + r"""
  const double lam = lame[0], mu = lame[1];
  double dl = 0.0, dm = 0.0;
  for (int r = 0; r < NRHS; ++r) {""" + _prism_prep("w", "w") + _prism_prep("u", "u") + r"""
    double Sxy[2][3][2] = {{{0}}}, T[3][3] = {{0}};
    for (int zq = 0; zq < 2; ++zq) {
      const double z1 = ZQ[zq], z0 = 1.0 - z1;
      for (int tq = 0; tq < 3; ++tq) {""" + _prism_grad("w") + _prism_grad("u") + r"""
        const double trw = wdu[0][0] + wdu[1][1] + wdu[2][2];
        const double tru = udu[0][0] + udu[1][1] + udu[2][2];
        double s[3][3], ee = 0.0;
        for (int c = 0; c < 3; ++c)
          for (int d = 0; d < 3; ++d) {
            const double ew = wdu[c][d] + wdu[d][c];
            s[c][d] = mu * ew + (c == d ? lam * trw : 0.0);
            ee += ew * (udu[c][d] + udu[d][c]);
          }
        dl += wq * trw * tru;
        dm += wq * 0.5 * ee;
        const double w0 = wq * z0, w1 = wq * z1;
        for (int c = 0; c < 3; ++c) {
          Sxy[0][c][0] += w0 * s[c][0]; Sxy[0][c][1] += w0 * s[c][1];
          Sxy[1][c][0] += w1 * s[c][0]; Sxy[1][c][1] += w1 * s[c][1];
          for (int a = 0; a < 3; ++a) T[a][c] += wq * TL[tq][a] * s[c][2];
        }
      }
    }
    for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c) {
        const double xy0 = g[a][0] * Sxy[0][c][0] + g[a][1] * Sxy[0][c][1];
        const double xy1 = g[a][0] * Sxy[1][c][0] + g[a][1] * Sxy[1][c][1];
        du[(a * NRHS + r) * 3 + c] += xy0 - T[a][c] * ih;
        du[((a + 3) * NRHS + r) * 3 + c] += xy1 + T[a][c] * ih;
      }
  }
  dlame[0] = dl;
  dlame[1] = dm;
}
#undef NRHS
""")

# 18 x 18 element stiffness matrix (3x3 blocks per node pair) into a BAIJ Mat.
PRISM_ELASTICITY_MATRIX = (r"""
static void prism_elasticity_mat(double A[18][18], const double *restrict X,
                                 const double *restrict lame)
{""" + _PRISM_GEOM + r"""
  const double lam = lame[0], mu = lame[1];
  double B[6][6][3][3];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j)
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) B[i][j][c][d] = 0.0;
  for (int zq = 0; zq < 2; ++zq) {
    const double z1 = ZQ[zq], z0 = 1.0 - z1;
    for (int tq = 0; tq < 3; ++tq) {
      double G[6][3];
      for (int a = 0; a < 3; ++a) {
        G[a][0] = g[a][0] * z0; G[a][1] = g[a][1] * z0; G[a][2] = -TL[tq][a] * ih;
        G[a + 3][0] = g[a][0] * z1; G[a + 3][1] = g[a][1] * z1; G[a + 3][2] = TL[tq][a] * ih;
      }
      double lG[6][3], mG[6][3];
      for (int i = 0; i < 6; ++i)
        for (int c = 0; c < 3; ++c) {
          lG[i][c] = wq * lam * G[i][c];
          mG[i][c] = wq * mu * G[i][c];
        }
      /* K is symmetric: the (i, j) block is the transpose of the (j, i)
         block, so only node pairs i <= j are computed */
      for (int i = 0; i < 6; ++i)
        for (int j = i; j < 6; ++j) {
          const double dot = mG[i][0] * G[j][0] + mG[i][1] * G[j][1] + mG[i][2] * G[j][2];
          for (int c = 0; c < 3; ++c)
            for (int d = 0; d < 3; ++d)
              B[i][j][c][d] += lG[i][c] * G[j][d] + mG[i][d] * G[j][c] + (c == d ? dot : 0.0);
        }
    }
  }
  for (int i = 0; i < 6; ++i)
    for (int j = i; j < 6; ++j)
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) {
          A[3 * i + c][3 * j + d] += B[i][j][c][d];
          if (j != i) A[3 * j + d][3 * i + c] += B[i][j][c][d];
        }
}
""")


def build_prisms(op2, n=256, layers=65, seed=0, nrhs=PRISM_NRHS):
    """Config 5: n x n split-square base extruded to `layers` levels
    (layers - 1 prisms per column), P1 displacement (nrhs, 3) per node,
    Lame (lambda, mu) per prism ~ lognormal(0, 0.3) (seeded)."""
    bc, tri, base, offset, nnodes, ncoords = meshes.extruded_prisms(n, layers, seed=seed)
    Cb = tri.shape[0]
    ncell = Cb * (layers - 1)
    rng = np.random.default_rng(seed + 5)
    bset = op2.Set(Cb, "base_cells")
    cells = op2.ExtrudedSet(bset, layers)
    nodes = op2.Set(nnodes, "nodes")
    prisms = op2.Set(ncell, "prisms")
    c2n = op2.Map(cells, nodes, 6, base, "cell2node", offset)
    c2c = op2.Map(cells, prisms, 1, (np.arange(Cb) * (layers - 1)).astype(np.int32), "cell2cell",
                  np.ones(1, dtype=np.int32))
    X = op2.Dat(nodes ** 3, ncoords, np.float64, "coords")
    lame = np.stack([rng.lognormal(0.0, 0.3, ncell), rng.lognormal(0.0, 0.3, ncell)], axis=1)
    L = op2.Dat(prisms ** 2, lame, np.float64, "lame")
    u = rng.uniform(-1, 1, (nnodes, nrhs, 3))
    w = rng.uniform(-1, 1, (nnodes, nrhs, 3))
    return dict(cells=cells, nodes=nodes, prisms=prisms, c2n=c2n, c2c=c2c, X=X, L=L,
                u=u, w=w, nrhs=nrhs, ncell=ncell, nnodes=nnodes)
