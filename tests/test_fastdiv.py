"""Division by invariant integers (Granlund & Montgomery, PLDI 1994) as the
sweep kernels use it (FastDiv in espins_gb300/csrc/esp_device.cuh): the
multiplier and shift restated here give n // d for every 0 <= n < 2^31."""
import random


def _make(d):
    l = 0
    while (1 << l) < d:
        l += 1
    m = ((((1 << l) - d) << 32) // d + 1) & 0xFFFFFFFF
    return (0 if d == 1 else m), l


def test_multiply_shift_division_is_exact():
    rng = random.Random(7)
    divisors = list(range(1, 300)) + [rng.randint(1, 1 << 24) for _ in range(2000)]
    for d in divisors:
        m, l = _make(d)
        for n in (0, 1, d - 1, d, d + 1, 2 * d - 1, (1 << 31) - 1, rng.randint(0, (1 << 31) - 1),
                  rng.randint(0, 1 << 16)):
            assert ((((n * m) >> 32) + n) >> l) == n // d, (n, d)
