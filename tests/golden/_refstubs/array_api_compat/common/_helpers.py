def device(x, /):
    return "cpu"
