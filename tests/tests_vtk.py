"""Test helper: write a restart VTK file in the reference's layout."""


def write_restart(path, values, nx, ny, spacing):
    head = ("# vtk DataFile Version 3.0\nDensity Data\nASCII\nDATASET STRUCTURED_POINTS\n"
            f"DIMENSIONS {nx} {ny} 1\nORIGIN 0 0 0\nSPACING {spacing} {spacing} 1\n"
            f"POINT_DATA {nx * ny}\nSCALARS DensityData float\nLOOKUP_TABLE default\n")
    with open(path, "w") as f:
        f.write(head + "".join(f"{v:.17g}\n" for v in values))
