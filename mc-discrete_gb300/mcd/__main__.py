"""python -m mcd -i input.file: run a whole simulation (mcd.doScatter.main)."""
from .doScatter import main

main()
