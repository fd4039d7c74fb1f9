"""Hartree atomic units used by the ldbd_data files and param.in.

The constants restate the values of the reference's ``comm/Units.h`` (JDFTx units header:
eV, Kelvin, fs, Tesla2au, bohr2cm) so that files written here are read by DMD with the same
numbers it would compute itself.
"""
import math

eV = 1.0 / 27.21138505
Joule = 1.0 / 4.35974434e-18
Kelvin = 1.3806488e-23 * Joule
Angstrom = 1.0 / 0.5291772
meter = 1e10 * Angstrom
kg = 1.0 / 9.10938291e-31
Newton = Joule / meter
sec = math.sqrt((kg * meter) / Newton)
fs = sec * 1.0e-15
ps = 1000.0 * fs
Tesla2au = 1.0 / 2.3505175675871e5
bohr2cm = 5.291772109038e-9
# a.u. of time -> ps, the conversion the reference's T1 fit script uses
AU_TO_PS = 2.4188843265857e-5
