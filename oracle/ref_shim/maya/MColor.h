/* Minimal stand-in for the Maya type named by util/math.h (test shim only). */
#pragma once
class MColor { public: enum MColorType { kRGB, kHSV }; float r, g, b, a; };
