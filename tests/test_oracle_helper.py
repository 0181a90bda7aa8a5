"""Port of test/test_helper.jl: the label shifts apply_MPO uses to wire an
MPO's tensors after the state's (src/helper.jl:6-17) and the power-of-two
check of MPS(psi) (src/helper.jl:24-27)."""
import oracle as O


def test_shift_pair():
    # test_helper.jl: step 5 moves tensor 1 to tensor 6, the leg unchanged
    assert O.shift_pair((1, 1), 5) == (6, 1)


def test_shift_summation():
    s1 = O.Summation([(1, 1), (6, 1)])
    s2 = O.Summation([(6, 1), (11, 1)])
    assert O.shift_summation(s1, 5) == s2


def test_is_power_two():
    # the reference draws N from 2:10; every N of that range here
    for n in range(2, 11):
        assert O.is_power_two(2 ** n)
        assert not O.is_power_two(2 ** n - 1)
    assert not O.is_power_two(0)
