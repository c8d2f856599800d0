dim = 1.0
