// Enumerations of the reference's public API (types.hpp:23-29), same values.
#ifndef CUDAPROB3_GB300_TYPES_HPP
#define CUDAPROB3_GB300_TYPES_HPP

namespace cudaprob3 {

enum ProbType : int {
    e_e = 0, e_m = 1, e_t = 2,
    m_e = 3, m_m = 4, m_t = 5,
    t_e = 6, t_m = 7, t_t = 8
};

enum NeutrinoType { Neutrino, Antineutrino };

}  // namespace cudaprob3

#endif
