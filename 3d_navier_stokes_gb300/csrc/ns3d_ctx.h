// ns3d_ctx.h — the context behind the C ABI's ns3d_ctx handle (internal).
#pragma once
#include "ns3d_base.h"

struct ns3d_ctx {
    ns3d_params p;
    ns3d::Base* impl;
    cudaStream_t stream;
    bool own_stream;
    char err[512];
};
