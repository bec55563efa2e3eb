class CPUDispatcher:  # only used in isinstance checks by the reference
    pass
