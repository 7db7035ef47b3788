// frames.hpp -- frame files of the command line (host code, no GPU).
//
// The reference reads and writes frames through iio (lib/iio); this library has
// no image libraries and reads and writes the formats its scripts use itself:
//   .pfm        Portable Float Map: "Pf" grey or "PF" three channels, rows
//               bottom to top, little endian when the scale is negative;
//   .tif/.tiff  baseline TIFF, uncompressed: read with 8-, 16- or 32-bit
//               unsigned integer or 32-bit float samples, 1 to 4 per pixel,
//               interleaved or planar, in strips, either byte order (values
//               taken as they are, as iio does); written as 32-bit float,
//               little endian, interleaved, one strip;
//   .flo        Middlebury optical flow: "PIEH", int32 width and height, then
//               interleaved (u, v) float32 pixels, top row first (the layout
//               iio reads, lib/iio/iio.c:1885-1903);
//   .png        output only: 8-bit grey or RGB, values rounded and clamped to
//               [0, 255], stored (uncompressed) deflate blocks.
// Any other extension is read and written as PFM.  As the reference's
// loadImage does (src/utils/lib_image.cpp:66-73), a three-channel frame whose
// channels are all equal is read as grey.  Frames are planar (c, y, x) floats.
#pragma once

#include <string>
#include <vector>

namespace bm4dof_frames {

bool read_frame(const char *path, std::vector<float> &out, int &w, int &h, int &c);

// A video as the command lines hold it: planar frames (c, y, x), frame after
// frame, like the reference's Video<float> (src/utils/lib_videot.hpp:134-181).
struct Video {
	std::vector<float> data;
	unsigned w = 0, h = 0, c = 0, f = 0;
};

// Video<float>::loadVideo (src/utils/lib_videot.cpp:30-89): frames first,
// first+step, ... up to last, named by the printf pattern; (last-first+1)/step
// frames; err receives the reference's message on failure.
bool load_video(const std::string &pattern, unsigned first, unsigned last, unsigned step, Video &v,
                std::string &err);

// Video<float>::saveVideo (src/utils/lib_videot.cpp:91-126): v.f frames named
// first, first+step, ..., written by write_frame (no clipping).
bool save_video(const std::string &pattern, unsigned first, unsigned step, const Video &v, std::string &err);
bool write_frame(const char *path, const float *planar, int w, int h, int c);

// One grey frame as the reference's optical-flow tool reads it
// (iio_read_image_float, lib/iio/iio.c:3486-3505): three channels become
// .299 r + .587 g + .114 b, and four (colour and alpha) the same of the first
// three, computed in double and stored in the file's sample type -- so
// truncated for integer samples -- before the conversion to float.  Other
// channel counts, and sample types iio does not reduce (32-bit integers, 16-bit
// with alpha), are refused with the reason in why.
bool read_grey(const char *path, std::vector<float> &out, int &w, int &h, std::string &why);

// A flow field (u plane, then v plane) as the optical-flow tool saves it: a
// two-channel float TIFF for .tif/.tiff names, Middlebury .flo for any other.
bool write_flow(const char *path, const float *uv, int w, int h);

}  // namespace bm4dof_frames
