"""2-D test cases shared by the oracle and GPU tests."""
import numpy as np


def cooks_membrane(tmp_path, n):
    """Cook's membrane as the reference's cooksMembrane tutorial meshes it
    (one blockMesh hex block, straight edges, n x n x 1, corners (0,0),
    (48,44), (48,60), (0,44) mm, 1 mm thick), with the empty front and back
    faces left out of the discretisation (2-D)."""
    from solids4foam_gb300.foam_case import polymesh_from_cells, read_case, write_polymesh
    V = np.array([[0, 0], [48, 44], [48, 60], [0, 44]], float) * 1e-3
    pid = lambda i, j, k: i + (n + 1) * (j + (n + 1) * k)
    pts = []
    for z in (-0.5e-3, 0.5e-3):
        for j in range(n + 1):
            for i in range(n + 1):
                s, t = i / n, j / n
                P = (1 - s) * (1 - t) * V[0] + s * (1 - t) * V[1] + s * t * V[2] + (1 - s) * t * V[3]
                pts.append([P[0], P[1], z])
    cells = []
    for j in range(n):
        for i in range(n):
            v = [pid(i, j, 0), pid(i + 1, j, 0), pid(i + 1, j + 1, 0), pid(i, j + 1, 0)]
            w = [pid(i, j, 1), pid(i + 1, j, 1), pid(i + 1, j + 1, 1), pid(i, j + 1, 1)]
            cells.append([v, w] + [[v[e], v[(e + 1) % 4], w[(e + 1) % 4], w[e]] for e in range(4)])

    def patch_of(c):
        if abs(abs(c[2]) - 0.5e-3) < 1e-12:
            return 3                                   # frontAndBack (empty)
        return 0 if abs(c[0]) < 1e-12 else 1 if abs(c[0] - 0.048) < 1e-12 else 2
    case = tmp_path / f"cook{n}"
    write_polymesh(str(case / "constant" / "polyMesh"),
                   **polymesh_from_cells(np.array(pts), cells, patch_of,
                                         ["left", "right", "topAndBottom", "frontAndBack"]))
    m, _ = read_case(str(case), d_file=None)
    nf = int(m["patch_start"][3])                      # frontAndBack is the last patch
    m2 = dict(owner=m["owner"][:nf], neighbour=m["neighbour"], C=m["C"], V=m["V"],
              Cf=m["Cf"][:nf], Sf=m["Sf"][:nf], patch_start=m["patch_start"][:3],
              patch_size=m["patch_size"][:3], patch_names=["left", "right", "topAndBottom"])
    return m, m2


def cooks_membrane_case(case, n, rotate_deg=0.0):
    """The cooksMembrane tutorial as a case directory: the polyMesh with
    frontAndBack of type empty, 0/D, constant/solidProperties and
    mechanicalProperties, system/fvSolution, as the tutorial sets them.
    rotate_deg turns the mesh about the x axis (empty patches then no longer
    normal to an axis)."""
    import pathlib
    from solids4foam_gb300.foam_case import polymesh_from_cells, write_polymesh
    case = pathlib.Path(case)
    V = np.array([[0, 0], [48, 44], [48, 60], [0, 44]], float) * 1e-3
    pid = lambda i, j, k: i + (n + 1) * (j + (n + 1) * k)
    pts = []
    for z in (-0.5e-3, 0.5e-3):
        for j in range(n + 1):
            for i in range(n + 1):
                s, t = i / n, j / n
                P = (1 - s) * (1 - t) * V[0] + s * (1 - t) * V[1] + s * t * V[2] + (1 - s) * t * V[3]
                pts.append([P[0], P[1], z])
    cells = []
    for j in range(n):
        for i in range(n):
            v = [pid(i, j, 0), pid(i + 1, j, 0), pid(i + 1, j + 1, 0), pid(i, j + 1, 0)]
            w = [pid(i, j, 1), pid(i + 1, j, 1), pid(i + 1, j + 1, 1), pid(i, j + 1, 1)]
            cells.append([v, w] + [[v[e], v[(e + 1) % 4], w[(e + 1) % 4], w[e]] for e in range(4)])

    def patch_of(c):
        if abs(abs(c[2]) - 0.5e-3) < 1e-12:
            return 3
        return 0 if abs(c[0]) < 1e-12 else 1 if abs(c[0] - 0.048) < 1e-12 else 2
    pm = polymesh_from_cells(np.array(pts), cells, patch_of,
                             ["left", "right", "topAndBottom", "frontAndBack"])
    if rotate_deg:
        a = np.radians(rotate_deg)
        R = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
        pm["points"] = pm["points"] @ R.T
    write_polymesh(str(case / "constant" / "polyMesh"), **pm,
                   patch_types=["patch", "patch", "patch", "empty"])
    head = "FoamFile { version 2.0; format ascii; class dictionary; object x; }\n"
    (case / "0").mkdir(exist_ok=True)
    (case / "0" / "D").write_text(head.replace("dictionary", "volVectorField") + """
dimensions [0 1 0 0 0 0 0];
internalField uniform (0 0 0);
boundaryField
{
    left { type fixedDisplacement; value uniform (0 0 0); }
    right { type solidTraction; traction uniform (0 6.25e6 0); pressure uniform 0; }
    topAndBottom { type solidTraction; traction uniform (0 0 0); pressure uniform 0; }
    frontAndBack { type empty; }
}
""")
    (case / "constant" / "solidProperties").write_text(head + """
solidModel linearGeometryTotalDisplacement;
"linearGeometryTotalDisplacementCoeffs|unsLinearGeometryCoeffs"
{ nCorrectors 5000; solutionTolerance 1e-07; alternativeTolerance 1e-07; infoFrequency 100; }
""")
    (case / "constant" / "mechanicalProperties").write_text(head + """
planeStress no;
mechanical ( steel { type linearElastic; rho rho [1 -3 0 0 0 0 0] 1;
                     E E [1 -1 -2 0 0 0 0] 70e6; nu nu [0 0 0 0 0 0 0] 0.3333; } );
""")
    (case / "system").mkdir(exist_ok=True)
    (case / "system" / "fvSolution").write_text(head + """
solvers { D { solver PCG; preconditioner FDIC; tolerance 1e-09; relTol 0.1; maxIter 200; } }
relaxationFactors { equations { } fields { } }
""")
    # the tutorial's gradient scheme (its system/fvSchemes, gradSchemes)
    (case / "system" / "fvSchemes").write_text(head + """
gradSchemes { default none; grad(D) extendedLeastSquares 0; }
""")
    return str(case)
