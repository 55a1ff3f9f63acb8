/* Minimal stand-in for the Maya type named by util/math.h (test shim only). */
#pragma once
class MMatrix {
public:
    double m[4][4];
    void get(float out[4][4]) const {
        for (int i = 0; i < 4; ++i) for (int j = 0; j < 4; ++j) out[i][j] = (float)m[i][j];
    }
};
