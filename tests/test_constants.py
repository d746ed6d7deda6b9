"""The device transforms use that ω_R = 7^((p−1)/R) is a power of two for R ≤ 64 (so a twiddle
of a sub-transform is a shift); these are the exponents the kernels are compiled with."""
P = 0xFFFFFFFF00000001
EXPONENTS = {2: 96, 4: 48, 8: 120, 16: 156, 32: 78, 64: 39}


def test_small_roots_are_powers_of_two():
    for r, e in EXPONENTS.items():
        assert pow(7, (P - 1) // r, P) == pow(2, e, P)
    assert pow(2, 192, P) == 1 and pow(2, 96, P) == P - 1
