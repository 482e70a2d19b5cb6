"""Derived physical quantities of a GlobalSimuState-shaped result, as MolFlow+'s CSV exporter
computes them (src/IO/CSVExporter.cpp), and its facet-physics table.

* molecules_per_tp  — GetMoleculesPerTP (CSVExporter.cpp:59-79): real molecules (per second)
  one test particle stands for: the final outgassing rate over the desorbed test particles in
  constant flow (moment 0), the total desorbed molecules over the window length per desorbed
  test particle in a time moment.
* density_correction — DensityCorrection (CSVExporter.cpp:85-107): 1 - (abs + des) / (hits + des) / 2
  on desorbing or absorbing facets, else 1.
* facet_quantities  — impingement rate, particle and mass density, pressure and mean molecular
  speed of every facet (CSVExporter.cpp:274-321), per cm^2 of facet area counted twice for a
  two-sided facet (GetArea, :110-112).
* write_facet_physics_csv — ExportPhysicalQuantitiesForFacets (CSVExporter.cpp:400-425): the
  columns "#", "Imping.rate", "Pressure [mbar]", "Density [1/m3]", "Density [kg/m3]",
  "Av.mol.speed[m/s]", one line per facet.

The column names, constants (1E4 cm^2 -> m^2, 6E23, 0.01 Pa -> mbar) and formulas are those of
the reference so that the tables read the same.
"""
import numpy as np

from . import _abi as A

PHYSICS_COLUMNS = ["#", "Imping.rate", "Pressure [mbar]", "Density [1/m3]", "Density [kg/m3]", "Av.mol.speed[m/s]"]


def molecules_per_tp(state, outgassing, moment=0, moment_windows=None):
    """GetMoleculesPerTP.  `outgassing` is GpuModel.outgassing() (CalcTotalOutgassing totals)."""
    n = float(state.global_[A.G_NBDESORBED])
    if n == 0:
        return 0.0
    if moment == 0:
        return outgassing["final_outgassing_rate"] / n
    return (outgassing["total_desorbed_molecules"] / float(moment_windows[moment - 1])) / n


def density_correction(n_mc_hit, n_desorbed, n_hit_equiv, n_abs_equiv):
    """DensityCorrection of each facet (arrays)."""
    n_mc_hit = np.asarray(n_mc_hit, np.float64)
    n_desorbed = np.asarray(n_desorbed, np.float64)
    n_hit_equiv = np.asarray(n_hit_equiv, np.float64)
    n_abs_equiv = np.asarray(n_abs_equiv, np.float64)
    active = ((n_mc_hit > 0) | (n_desorbed > 0)) & ((n_abs_equiv > 0) | (n_desorbed > 0))
    den = np.where(active, n_hit_equiv + n_desorbed, 1.0)
    return np.where(active, 1.0 - (n_abs_equiv + n_desorbed) / den / 2.0, 1.0)


def facet_quantities(model, state, area, outgassing, moment=0):
    """Per-facet impingement rate [1/m2/s], particle density [1/m3], mass density [kg/m3],
    pressure [mbar] and mean molecular speed [m/s] of moment block `moment`.  `area` is the facet
    area in cm^2 (GpuModel.facet_geometry()[1])."""
    fc = state.facet_counts[moment].astype(np.float64)
    fs = state.facet_sums[moment]
    sides = np.where(np.asarray(model.is_2sided) != 0, 2.0, 1.0)
    a = np.asarray(area, np.float64) * sides
    mol = molecules_per_tp(state, outgassing, moment, getattr(model, "moment_window", None))
    hit_equiv = fs[:, A.FS_NBHITEQUIV]
    corr = density_correction(fc[:, A.FC_NBMCHIT], fc[:, A.FC_NBDESORBED], hit_equiv, fs[:, A.FS_NBABSEQUIV])
    mass = float(model.gas_mass) / 1000.0 / 6e23
    impingement = hit_equiv / a * (1e4 * mol)
    density = fs[:, A.FS_SUM_1_PER_ORT_VEL] / a * (1e4 * mol) * corr
    s1v = fs[:, A.FS_SUM_1_PER_VELOCITY]
    speed = np.where(s1v == 0.0, 0.0, (hit_equiv + fc[:, A.FC_NBDESORBED]) / np.where(s1v == 0.0, 1.0, s1v))
    return {
        "impingement_rate": impingement,
        "density_1p": density,
        "density_kgp": density * mass,
        "pressure_mbar": fs[:, A.FS_SUM_V_ORT] * (1e4 * mol * mass * 0.01) / a,
        "avg_speed": speed,
    }


def pressure_per_sum_v_ort(model, area, outgassing, facets):
    """Factor turning Sum v_ort per desorbed test particle on each of `facets` into its constant-flow
    pressure in mbar: pressure = factor * (Sum v_ort / desorptions).  (GetMoleculesPerTP times the
    desorption count is the final outgassing rate, so the count cancels.)"""
    facets = np.asarray(facets)
    sides = np.where(np.asarray(model.is_2sided)[facets] != 0, 2.0, 1.0)
    mass = float(model.gas_mass) / 1000.0 / 6e23
    return outgassing["final_outgassing_rate"] * 1e4 * mass * 0.01 / (np.asarray(area, np.float64)[facets] * sides)


def _fmt(x):
    """A value as fmt's "{}" prints it: the shortest round-trip form, integral doubles without '.0'."""
    if isinstance(x, (int, np.integer)):
        return str(int(x))
    r = repr(float(x))
    return r[:-2] if r.endswith(".0") else r


def facet_physics_table(model, state, area, outgassing, moment=0):
    """The facet-physics table as text (header line, then one line per facet)."""
    q = facet_quantities(model, state, area, outgassing, moment)
    lines = [",".join(PHYSICS_COLUMNS)]
    for i in range(model.n_facets):
        lines.append(",".join([_fmt(i + 1), _fmt(q["impingement_rate"][i]), _fmt(q["pressure_mbar"][i]),
                               _fmt(q["density_1p"][i]), _fmt(q["density_kgp"][i]), _fmt(q["avg_speed"][i])]))
    return "\n".join(lines) + "\n"


def write_facet_physics_csv(path, model, state, area, outgassing, moment=0):
    """ExportPhysicalQuantitiesForFacets: write the table to `path`; returns 0, or 1 when the file
    cannot be written (the reference's convention)."""
    try:
        with open(path, "w") as f:
            f.write(facet_physics_table(model, state, area, outgassing, moment))
    except OSError:
        return 1
    return 0


def validate_csv(path):
    """ValidateCSVFile (CSVExporter.cpp:431-448): the number of separators per line when every
    line has the same, -1 for an empty file, -2 for a ragged one."""
    try:
        with open(path) as f:
            lines = f.read().splitlines()
    except OSError:
        return -1
    if not lines:
        return -1
    n = lines[0].count(",")
    return n if all(ln.count(",") == n for ln in lines[1:]) else -2
