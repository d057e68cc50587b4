// mlp_layout.h -- parameter layout of the dispatcher's MLP, shared by inference and training.
#pragma once

#include <cstdint>

namespace galp {

// Sizes of the MLP parameter block: W1[nin][nhid], b1[nhid], W2[nhid][nhid], b2[nhid],
// W3[nhid][nout], b3[nout] (row-major, input index first).
inline int64_t mlp_param_count(int nin, int nhid, int nout)
{
    return (int64_t)nin * nhid + nhid + (int64_t)nhid * nhid + nhid + (int64_t)nhid * nout + nout;
}

}  // namespace galp
