// super_resolution_kv2: capture/super_resolution_kv2/super_resolution_kv2.cpp,
// Kinect v2 (float depth stored as 8-bit RGBA PNGs); the body is sr_tool::run.
#include "sr_tool.h"

int main(int argc, char* argv[]) { return sr_tool::run(argc, argv, true); }
