def profile(func=None, **_kw):
    return func if func is not None else (lambda f: f)
