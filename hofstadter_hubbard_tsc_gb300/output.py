"""Measurement output files in the reference's text formats.

Data records use the reference's edit descriptors exactly; a field that does
not fit its width is filled with asterisks, as Fortran formatted output does.
Header records are list-directed in the reference (write(u,*)), whose spacing
differs between Fortran compilers; they are written here in gfortran's
layout (a leading blank, integers in 12 columns, reals in 25 columns) and
carry the same tokens in the same order (reals with 16 decimals), so
whitespace-splitting readers see the same fields.

  * num_elec.dat (measure_operator_dia, code/measure.f90:43-56): header, then
    per site format (2i6, 3f14.8): x, y, <O_i>, running sum; a blank record;
    appended.
  * spin_cor.dat, elec_cor.dat, density_cor.dat (code/quantum.f90:514-559):
    header, then for every nonzero entry format (3i8, 3f21.14):
    i, j, (j-1)/W - (i-1)/W, Re C_ij, Im C_ij (density: Re C_ij, <n_i>,
    <n_j>); the file is rewritten.
  * strfac_*.dat (Get_structure_factor_cut, code/measure.f90:2211-2219):
    header, then format (F16.12,1X,F16.12,1X,F16.12): kx/pi, ky/pi, S with
    kx running fastest; a blank record; appended.
"""
import numpy as np


def _field(text, width):
    return "*" * width if len(text) > width else text.rjust(width)


def fortran_i(n, width):
    """Iw."""
    return _field(str(int(n)), width)


def fortran_f(x, width, decimals):
    """Fw.d.  The decimal conversion is Python's correctly rounded one; it can
    differ from a Fortran runtime's only for a value exactly halfway between
    two printable decimals."""
    return _field(f"{float(x):.{decimals}f}", width)


def list_directed(*items):
    """One list-directed record in gfortran's layout: a string that follows a
    number is separated from it by a blank."""
    out = []
    after_number = False
    for it in items:
        if isinstance(it, str):
            out.append((" " if after_number else "") + it)
            after_number = False
        elif isinstance(it, (int, np.integer)):
            out.append(f"{int(it):12d}")
            after_number = True
        else:
            out.append(f"{float(it):25.16f}")
            after_number = True
    return " " + "".join(out)


def write_site_profile(path, prof, W, n_up, n_down, kept_min, kept_max):
    """measure_operator_dia's record of <O_i> (appended)."""
    L = len(prof) // W
    lines = [list_directed("Nx=", L, "Ny=", W, "N_up=", n_up, "N_down=", n_down, "M1=", kept_min, "M2=", kept_max)]
    total = 0.0
    for i, v in enumerate(np.real(np.asarray(prof)), start=1):
        total += v
        lines.append(fortran_i((i - 1) // W + 1, 6) + fortran_i((i - 1) % W + 1, 6) + fortran_f(v, 14, 8)
                     + fortran_f(total, 14, 8))
    lines.append(" ")
    with open(path, "a") as f:
        f.write("\n".join(lines) + "\n")


def write_correlations(path, corr, W, J2, kept_max, density=None):
    """spin_cor.dat / elec_cor.dat (density None) or density_cor.dat (density
    = <n_i>): every nonzero C_ij, the file rewritten."""
    C = np.asarray(corr, dtype=np.complex128)
    N = C.shape[0]
    lines = [list_directed("Nx=", N // W, "Ny=", W, "J2=", float(J2), "kept_max=", kept_max)]
    for i in range(1, N + 1):
        for j in range(1, N + 1):
            c = C[i - 1, j - 1]
            if abs(c) == 0.0:
                continue
            head = fortran_i(i, 8) + fortran_i(j, 8) + fortran_i((j - 1) // W - (i - 1) // W, 8)
            if density is None:
                tail = fortran_f(c.real, 21, 14) + fortran_f(c.imag, 21, 14)
            else:
                tail = (fortran_f(c.real, 21, 14) + fortran_f(np.real(density[i - 1]), 21, 14)
                        + fortran_f(np.real(density[j - 1]), 21, 14))
            lines.append(head + tail)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_structure_factor(path, kx, ky, S, W, L, n_up, n_down, kept_min, kept_max):
    """Get_structure_factor_cut's record (appended); kx, ky in units of pi,
    S indexed [kx, ky] as measure.structure_factor returns it."""
    lines = [list_directed("Nx=", L, "Ny=", W, "N_up=", n_up, "N_down=", n_down, "M1=", kept_min, "M2=", kept_max)]
    for j in range(len(ky)):
        for i in range(len(kx)):
            lines.append(fortran_f(kx[i], 16, 12) + " " + fortran_f(ky[j], 16, 12) + " " + fortran_f(S[i, j], 16, 12))
    lines.append(" ")
    with open(path, "a") as f:
        f.write("\n".join(lines) + "\n")
