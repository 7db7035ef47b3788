// frames_convert.cpp -- TEST DRIVER: reads one frame file with the command
// line's reader and writes it with its writer (formats by extension), so that
// tests/test_frames.py can check frames.cpp without a GPU.
#include <cstdio>
#include <vector>

#include "../bm4d-of_gb300/csrc/frames.hpp"

int main(int argc, char **argv)
{
	if (argc != 3) return 2;
	std::vector<float> v;
	int w = 0, h = 0, c = 0;
	if (!bm4dof_frames::read_frame(argv[1], v, w, h, c)) return 3;
	std::printf("%d %d %d\n", w, h, c);
	return bm4dof_frames::write_frame(argv[2], v.data(), w, h, c) ? 0 : 4;
}
