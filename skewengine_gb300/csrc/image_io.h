// Internal image input shared by the PNG reader and run(argc, argv).  Not part
// of the public ABI (include/skewengine.h).
#pragma once

#include <vector>

namespace ske {

// The reference's image input (helper::read_png, src/helper.h:167-184): the PNG
// decoded to 8-bit RGBA, then R + G + B per pixel as one float per cell.  The
// grid is sized only after the file has decoded, so a damaged file cannot make
// the caller allocate for the size its header claims.  SKE_OK or
// SKE_ERR_INVALID.
int png_read_grid(const char* path, int* width, int* height, std::vector<float>& grid);

// Record `msg` as the calling thread's last error (ske_last_error) and return
// `code` (defined with the engine's entry points).
int set_last_error(int code, const char* msg);

}  // namespace ske
