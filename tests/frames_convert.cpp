// frames_convert.cpp -- TEST DRIVER: reads one frame file with the command
// line's reader and writes it with its writer (formats by extension), so that
// tests/test_frames.py can check frames.cpp without a GPU.
//
//   frames_convert in out           read_frame, then write_frame
//   frames_convert -grey in out     read_grey (the optical-flow tool's reader),
//                                   then write_frame of the grey frame
//   frames_convert -flow in out     read_frame of a two-channel frame, then
//                                   write_flow
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../bm4d-of_gb300/csrc/frames.hpp"

int main(int argc, char **argv)
{
	const bool grey = argc == 4 && !std::strcmp(argv[1], "-grey");
	const bool flow = argc == 4 && !std::strcmp(argv[1], "-flow");
	if (argc != 3 && !grey && !flow) return 2;
	const char *in = argv[argc - 2], *out = argv[argc - 1];
	std::vector<float> v;
	int w = 0, h = 0, c = 1;
	if (grey) {
		std::string why;
		if (!bm4dof_frames::read_grey(in, v, w, h, why)) return std::fprintf(stderr, "%s\n", why.c_str()), 3;
	} else if (!bm4dof_frames::read_frame(in, v, w, h, c)) {
		return 3;
	}
	std::printf("%d %d %d\n", w, h, c);
	if (flow) return c == 2 && bm4dof_frames::write_flow(out, v.data(), w, h) ? 0 : 4;
	return bm4dof_frames::write_frame(out, v.data(), w, h, c) ? 0 : 4;
}
