"""Golden fixtures made from the reference's own code (make_golden.py) and their loaders."""
