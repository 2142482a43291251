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
