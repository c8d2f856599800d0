eV = 1.602176634e-19
KeV = 1e3 * eV
