m = 1.0
cm = 1e-2
nm = 1e-9
angstrom = 1e-10
