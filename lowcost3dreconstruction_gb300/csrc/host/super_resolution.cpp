// super_resolution: capture/super_resolution/super_resolution.cpp, Kinect v1
// (16-bit depth PNGs); the body is sr_tool::run.
#include "sr_tool.h"

int main(int argc, char* argv[]) { return sr_tool::run(argc, argv, false); }
