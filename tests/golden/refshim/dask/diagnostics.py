class ProgressBar:
    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False
