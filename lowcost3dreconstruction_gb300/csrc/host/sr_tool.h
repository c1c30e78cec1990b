// Shared body of the super_resolution and super_resolution_kv2 tools.
#pragma once

namespace sr_tool {

// Runs the tool on argv; kv2 selects the Kinect v2 file formats.  Returns the
// process exit status.
int run(int argc, char* argv[], bool kv2);

}  // namespace sr_tool
