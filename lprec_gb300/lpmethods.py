def fbp(*a, **k):
    raise NotImplementedError
