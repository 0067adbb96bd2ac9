// Stand-in for the generated ReyesConfig.h: the one option that
// src/base/Projection.cpp reads, set by the oracle's pin driver.
#pragma once
struct ReyesConfigStandIn {
    float ribbon = 32.0f;
    float cull_ribbon() const { return ribbon; }
};
extern ReyesConfigStandIn reyes_config;
