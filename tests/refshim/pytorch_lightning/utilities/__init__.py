def rank_zero_info(*a, **k):
    return None
