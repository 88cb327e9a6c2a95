// Stand-in for RandomGenerator (src/auxilliary/parallel_random.hh): the one
// virtual the adapter calls.
#pragma once
class RandomGenerator {
public:
    virtual ~RandomGenerator() = default;
    virtual double draw_uniform_real() = 0;
};
