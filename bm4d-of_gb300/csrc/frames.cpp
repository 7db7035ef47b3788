// frames.cpp -- frame files of the command line: PFM, TIFF, .flo, PNG
// (formats and conventions in frames.hpp).
#include "frames.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace bm4dof_frames {

namespace {

bool ends_with(const std::string &s, const char *e)
{
	const size_t n = std::strlen(e);
	return s.size() >= n && !s.compare(s.size() - n, n, e);
}

bool host_little_endian()
{
	const uint16_t v = 1;
	unsigned char b[2];
	std::memcpy(b, &v, 2);
	return b[0] == 1;
}

void swap4(unsigned char *p)
{
	std::swap(p[0], p[3]);
	std::swap(p[1], p[2]);
}

// bytes from the current position to the end of the file: a corrupt header
// cannot ask for more memory than the file holds
size_t remaining(FILE *f)
{
	const long here = std::ftell(f);
	if (here < 0 || std::fseek(f, 0, SEEK_END) != 0) return 0;
	const long end = std::ftell(f);
	std::fseek(f, here, SEEK_SET);
	return end > here ? (size_t)(end - here) : 0;
}

// planar (c, y, x) floats
bool read_pfm(const char *path, std::vector<float> &out, int &w, int &h, int &c)
{
	FILE *f = std::fopen(path, "rb");
	if (!f) return false;
	char tag[3] = {0, 0, 0};
	float scale = 0.f;
	bool ok = std::fscanf(f, "%2s %d %d %f", tag, &w, &h, &scale) == 4 && w > 0 && h > 0;
	if (ok) ok = std::fgetc(f) != EOF;   // the single whitespace before the data
	c = tag[1] == 'F' ? 3 : 1;
	ok = ok && tag[0] == 'P' && (tag[1] == 'F' || tag[1] == 'f');
	std::vector<unsigned char> raw;
	if (ok) ok = (size_t)w * h * c * 4 <= remaining(f);
	if (ok) {
		raw.resize((size_t)w * h * c * 4);
		ok = std::fread(raw.data(), 1, raw.size(), f) == raw.size();
	}
	std::fclose(f);
	if (!ok) return false;
	const bool swap = (scale < 0.f) != host_little_endian();
	out.assign((size_t)w * h * c, 0.f);
	for (int y = 0; y < h; y++)
		for (int x = 0; x < w; x++)
			for (int k = 0; k < c; k++) {
				unsigned char *p = &raw[(((size_t)(h - 1 - y) * w + x) * c + k) * 4];   // bottom row first
				if (swap) swap4(p);
				std::memcpy(&out[((size_t)k * h + y) * w + x], p, 4);
			}
	return true;
}

bool write_pfm(const char *path, const float *planar, int w, int h, int c)
{
	FILE *f = std::fopen(path, "wb");
	if (!f) return false;
	std::fprintf(f, "%s\n%d %d\n%s\n", c == 3 ? "PF" : "Pf", w, h, host_little_endian() ? "-1.0" : "1.0");
	std::vector<float> row((size_t)w * c);
	bool ok = true;
	for (int y = h - 1; y >= 0 && ok; y--) {
		for (int x = 0; x < w; x++)
			for (int k = 0; k < c; k++) row[(size_t)x * c + k] = planar[((size_t)k * h + y) * w + x];
		ok = std::fwrite(row.data(), sizeof(float), row.size(), f) == row.size();
	}
	return std::fclose(f) == 0 && ok;
}

bool read_flo(const char *path, std::vector<float> &out, int &w, int &h, int &c)
{
	FILE *f = std::fopen(path, "rb");
	if (!f) return false;
	float magic = 0.f;
	int32_t wh[2] = {0, 0};
	bool ok = std::fread(&magic, 4, 1, f) == 1 && std::fread(wh, 4, 2, f) == 2 && magic == 202021.25f &&
	          wh[0] > 0 && wh[1] > 0;
	w = wh[0];
	h = wh[1];
	c = 2;
	std::vector<float> raw;
	if (ok) ok = (size_t)w * h * 2 * sizeof(float) <= remaining(f);
	if (ok) {
		raw.resize((size_t)w * h * 2);
		ok = std::fread(raw.data(), sizeof(float), raw.size(), f) == raw.size();
	}
	std::fclose(f);
	if (!ok) return false;
	out.assign(raw.size(), 0.f);
	for (size_t p = 0; p < (size_t)w * h; p++) {
		out[p] = raw[2 * p];
		out[(size_t)w * h + p] = raw[2 * p + 1];
	}
	return true;
}

bool write_flo(const char *path, const float *planar, int w, int h)
{
	FILE *f = std::fopen(path, "wb");
	if (!f) return false;
	const float magic = 202021.25f;
	const int32_t wh[2] = {w, h};
	std::vector<float> raw((size_t)w * h * 2);
	for (size_t p = 0; p < (size_t)w * h; p++) {
		raw[2 * p] = planar[p];
		raw[2 * p + 1] = planar[(size_t)w * h + p];
	}
	bool ok = std::fwrite(&magic, 4, 1, f) == 1 && std::fwrite(wh, 4, 2, f) == 2 &&
	          std::fwrite(raw.data(), sizeof(float), raw.size(), f) == raw.size();
	return std::fclose(f) == 0 && ok;
}

uint32_t crc32(const unsigned char *p, size_t n, uint32_t c = 0xffffffffu)
{
	for (size_t i = 0; i < n; i++) {
		c ^= p[i];
		for (int k = 0; k < 8; k++) c = (c >> 1) ^ (0xedb88320u & (0u - (c & 1u)));
	}
	return c;
}

void put32(std::vector<unsigned char> &v, uint32_t x)
{
	for (int s = 24; s >= 0; s -= 8) v.push_back((unsigned char)(x >> s));
}

bool write_png(const char *path, const float *planar, int w, int h, int c)
{
	// scanlines: filter byte 0, then 8-bit samples
	const int cc = c == 3 ? 3 : 1;
	std::vector<unsigned char> raw;
	raw.reserve((size_t)h * (w * cc + 1));
	for (int y = 0; y < h; y++) {
		raw.push_back(0);
		for (int x = 0; x < w; x++)
			for (int k = 0; k < cc; k++) {
				float v = std::round(planar[((size_t)k * h + y) * w + x]);
				v = v < 0.f ? 0.f : (v > 255.f ? 255.f : v);
				raw.push_back((unsigned char)v);
			}
	}
	// zlib stream of stored blocks
	std::vector<unsigned char> z = {0x78, 0x01};
	uint32_t a = 1, b = 0;
	for (unsigned char ch : raw) {
		a = (a + ch) % 65521u;
		b = (b + a) % 65521u;
	}
	for (size_t o = 0; o < raw.size() || raw.empty();) {
		const size_t n = std::min<size_t>(65535, raw.size() - o);
		const bool last = o + n == raw.size();
		z.push_back(last ? 1 : 0);
		z.push_back((unsigned char)(n & 0xff));
		z.push_back((unsigned char)(n >> 8));
		z.push_back((unsigned char)(~n & 0xff));
		z.push_back((unsigned char)((~n >> 8) & 0xff));
		z.insert(z.end(), raw.begin() + o, raw.begin() + o + n);
		o += n;
		if (last) break;
	}
	put32(z, (b << 16) | a);
	std::vector<unsigned char> png = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n'};
	auto chunk = [&png](const char *type, const std::vector<unsigned char> &data) {
		put32(png, (uint32_t)data.size());
		std::vector<unsigned char> td(type, type + 4);
		td.insert(td.end(), data.begin(), data.end());
		png.insert(png.end(), td.begin(), td.end());
		put32(png, crc32(td.data(), td.size()) ^ 0xffffffffu);
	};
	std::vector<unsigned char> ihdr;
	put32(ihdr, (uint32_t)w);
	put32(ihdr, (uint32_t)h);
	ihdr.push_back(8);
	ihdr.push_back(cc == 3 ? 2 : 0);
	ihdr.push_back(0);
	ihdr.push_back(0);
	ihdr.push_back(0);
	chunk("IHDR", ihdr);
	chunk("IDAT", z);
	chunk("IEND", {});
	FILE *f = std::fopen(path, "wb");
	if (!f) return false;
	const bool ok = std::fwrite(png.data(), 1, png.size(), f) == png.size();
	return std::fclose(f) == 0 && ok;
}

// ---- TIFF (baseline, uncompressed) -------------------------------------------
struct TiffReader {
	const std::vector<unsigned char> &b;
	bool le;
	uint32_t u16(size_t o) const
	{
		if (o + 2 > b.size()) return 0;
		return le ? (uint32_t)b[o] | (uint32_t)b[o + 1] << 8 : (uint32_t)b[o] << 8 | (uint32_t)b[o + 1];
	}
	uint32_t u32(size_t o) const
	{
		if (o + 4 > b.size()) return 0;
		return le ? (uint32_t)b[o] | (uint32_t)b[o + 1] << 8 | (uint32_t)b[o + 2] << 16 | (uint32_t)b[o + 3] << 24
		          : (uint32_t)b[o] << 24 | (uint32_t)b[o + 1] << 16 | (uint32_t)b[o + 2] << 8 | (uint32_t)b[o + 3];
	}
	// values of one IFD entry (SHORT or LONG, inline or at an offset)
	std::vector<uint32_t> values(size_t e) const
	{
		const uint32_t type = u16(e + 2), count = u32(e + 4);
		std::vector<uint32_t> v;
		const size_t sz = type == 3 ? 2 : 4;
		if ((type != 3 && type != 4) || count == 0 || count > (1u << 24)) return v;
		const size_t base = sz * count <= 4 ? e + 8 : u32(e + 8);
		if (base + sz * (size_t)count > b.size()) return v;
		for (uint32_t i = 0; i < count; i++) v.push_back(type == 3 ? u16(base + 2 * i) : u32(base + 4 * i));
		return v;
	}
};

// *sample (if given) receives the sample type: 8, 16 or 32 for unsigned
// integers, 0 for 32-bit float
bool read_tiff(const char *path, std::vector<float> &out, int &w, int &h, int &c, int *sample = nullptr)
{
	FILE *f = std::fopen(path, "rb");
	if (!f) return false;
	std::vector<unsigned char> b;
	unsigned char buf[65536];
	size_t n;
	while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) b.insert(b.end(), buf, buf + n);
	std::fclose(f);
	if (b.size() < 8 || !((b[0] == 'I' && b[1] == 'I') || (b[0] == 'M' && b[1] == 'M'))) return false;
	const TiffReader r{b, b[0] == 'I'};
	if (r.u16(2) != 42) return false;
	const size_t ifd = r.u32(4);
	const uint32_t ne = r.u16(ifd);
	if (ifd + 2 + 12 * (size_t)ne > b.size()) return false;
	uint32_t width = 0, height = 0, spp = 1, comp = 1, planar = 1, rps = 0xffffffffu, fmt = 1;
	std::vector<uint32_t> bps, offs, counts;
	for (uint32_t i = 0; i < ne; i++) {
		const size_t e = ifd + 2 + 12 * (size_t)i;
		const uint32_t tag = r.u16(e);
		const std::vector<uint32_t> v = r.values(e);
		if (v.empty()) continue;
		switch (tag) {
		case 256: width = v[0]; break;
		case 257: height = v[0]; break;
		case 258: bps = v; break;
		case 259: comp = v[0]; break;
		case 273: offs = v; break;
		case 277: spp = v[0]; break;
		case 278: rps = v[0]; break;
		case 279: counts = v; break;
		case 284: planar = v[0]; break;
		case 339: fmt = v[0]; break;
		default: break;
		}
	}
	const uint32_t bits = bps.empty() ? 1 : bps[0];
	if (width == 0 || height == 0 || comp != 1 || spp < 1 || spp > 4 || offs.empty() ||
	    offs.size() != counts.size() || (planar != 1 && planar != 2))
		return false;
	if (!((fmt == 1 && (bits == 8 || bits == 16 || bits == 32)) || (fmt == 3 && bits == 32))) return false;
	for (uint32_t s : bps)
		if (s != bits) return false;
	w = (int)width;
	h = (int)height;
	c = (int)spp;
	if (sample) *sample = fmt == 3 ? 0 : (int)bits;
	const size_t bytes = bits / 8, wh = (size_t)w * h;
	if (wh * c * bytes > b.size()) return false;   // more samples than the file holds
	// the strips, in order, hold the samples in file order
	std::vector<unsigned char> data;
	data.reserve(wh * c * bytes);
	for (size_t s = 0; s < offs.size(); s++) {
		if ((size_t)offs[s] + counts[s] > b.size()) return false;
		data.insert(data.end(), b.begin() + offs[s], b.begin() + offs[s] + counts[s]);
	}
	if (data.size() < wh * c * bytes) return false;
	(void)rps;
	out.assign(wh * c, 0.f);
	const TiffReader d{data, r.le};
	for (size_t i = 0; i < wh * c; i++) {
		// sample i in file order -> (channel, pixel)
		const size_t k = planar == 1 ? i % c : i / wh, p = planar == 1 ? i / c : i % wh;
		float v;
		if (bits == 8) {
			v = (float)data[i];
		} else if (bits == 16) {
			v = (float)d.u16(2 * i);
		} else {
			const uint32_t u = d.u32(4 * i);
			if (fmt == 3) std::memcpy(&v, &u, 4);
			else v = (float)u;
		}
		out[k * wh + p] = v;
	}
	return true;
}

bool write_tiff(const char *path, const float *planar, int w, int h, int c)
{
	const size_t wh = (size_t)w * h, nbytes = wh * c * 4;
	std::vector<unsigned char> t;
	auto p16 = [&t](uint32_t x) { t.push_back((unsigned char)(x & 0xff)); t.push_back((unsigned char)(x >> 8)); };
	auto p32 = [&t](uint32_t x) { for (int s = 0; s < 32; s += 8) t.push_back((unsigned char)(x >> s)); };
	const int ne = 11;
	const uint32_t ifd = 8, extra = ifd + 2 + 12 * ne + 4;   // bits-per-sample and sample-format arrays
	const uint32_t data_off = extra + 2 * 4 * 2;
	t.insert(t.end(), {'I', 'I'});
	p16(42);
	p32(ifd);
	p16(ne);
	auto entry = [&](uint32_t tag, uint32_t type, uint32_t count, uint32_t value) {
		p16(tag);
		p16(type);
		p32(count);
		if (type == 3 && count == 1) { p16(value); p16(0); }
		else p32(value);
	};
	const bool many = c > 2;   // more than two SHORTs do not fit in the entry
	entry(256, 4, 1, (uint32_t)w);
	entry(257, 4, 1, (uint32_t)h);
	if (c == 1) entry(258, 3, 1, 32);
	else if (!many) entry(258, 3, 2, 32u | 32u << 16);
	else entry(258, 3, (uint32_t)c, extra);
	entry(259, 3, 1, 1);                               // no compression
	entry(262, 3, 1, c >= 3 ? 2 : 1);                  // RGB or black is zero
	entry(273, 4, 1, data_off);
	entry(277, 3, 1, (uint32_t)c);
	entry(278, 4, 1, (uint32_t)h);                     // one strip
	entry(279, 4, 1, (uint32_t)nbytes);
	entry(284, 3, 1, 1);                               // interleaved
	if (c == 1) entry(339, 3, 1, 3);
	else if (!many) entry(339, 3, 2, 3u | 3u << 16);
	else entry(339, 3, (uint32_t)c, extra + 8);
	p32(0);                                            // no next IFD
	for (int k = 0; k < 4; k++) p16(32);
	for (int k = 0; k < 4; k++) p16(3);
	const size_t head = t.size();
	t.resize(head + nbytes);
	for (size_t p = 0; p < wh; p++)
		for (int k = 0; k < c; k++) {
			uint32_t u;
			std::memcpy(&u, &planar[(size_t)k * wh + p], 4);
			unsigned char *q = &t[head + (p * c + k) * 4];
			for (int s = 0; s < 4; s++) q[s] = (unsigned char)(u >> (8 * s));
		}
	FILE *f = std::fopen(path, "wb");
	if (!f) return false;
	const bool ok = std::fwrite(t.data(), 1, t.size(), f) == t.size();
	return std::fclose(f) == 0 && ok;
}

}  // namespace

bool read_frame(const char *path, std::vector<float> &out, int &w, int &h, int &c)
{
	const std::string p(path);
	const bool tif = ends_with(p, ".tif") || ends_with(p, ".tiff") || ends_with(p, ".TIF") || ends_with(p, ".TIFF");
	bool ok = ends_with(p, ".flo") ? read_flo(path, out, w, h, c)
	          : tif                ? read_tiff(path, out, w, h, c)
	                               : read_pfm(path, out, w, h, c);
	if (ok && c == 3) {   // equal channels: grey (lib_image.cpp:66-73)
		const size_t wh = (size_t)w * h;
		size_t k = 0;
		while (k < wh && out[k] == out[wh + k] && out[k] == out[2 * wh + k]) k++;
		if (k == wh) {
			out.resize(wh);
			c = 1;
		}
	}
	return ok;
}

bool load_video(const std::string &pattern, unsigned first, unsigned last, unsigned step, Video &v,
                std::string &err)
{
	char name[1024];
	std::snprintf(name, sizeof name, pattern.c_str(), first);
	std::vector<float> frame;
	int w, h, c;
	if (!read_frame(name, frame, w, h, c)) {
		err = "Video<T>::loadVideo: loading of " + std::string(name) + " failed";
		return false;
	}
	v.w = w;
	v.h = h;
	v.c = c;
	v.f = (last - first + 1) / step;
	v.data.assign((size_t)v.w * v.h * v.c * v.f, 0.f);
	size_t o = 0;
	std::copy(frame.begin(), frame.end(), v.data.begin());
	o += frame.size();
	for (unsigned t = first + step; t <= last; t += step) {
		std::snprintf(name, sizeof name, pattern.c_str(), t);
		if (!read_frame(name, frame, w, h, c)) {
			err = "Video<T>::loadVideo: loading of " + std::string(name) + " failed";
			return false;
		}
		if ((unsigned)w != v.w || (unsigned)h != v.h || (unsigned)c != v.c) {
			err = "Video<T>::loadVideo: size of " + std::string(name) + " does not match video size";
			return false;
		}
		if (o + frame.size() > v.data.size()) v.data.resize(o + frame.size());
		std::copy(frame.begin(), frame.end(), v.data.begin() + o);
		o += frame.size();
	}
	return true;
}

bool save_video(const std::string &pattern, unsigned first, unsigned step, const Video &v, std::string &err)
{
	const size_t whc = (size_t)v.w * v.h * v.c;
	for (unsigned k = 0; k < v.f; k++) {
		char name[1024];
		std::snprintf(name, sizeof name, pattern.c_str(), first + k * step);
		if (!write_frame(name, v.data.data() + k * whc, v.w, v.h, v.c)) {
			err = "Video<T>::saveVideo: writing of " + std::string(name) + " failed";
			return false;
		}
	}
	return true;
}

bool read_grey(const char *path, std::vector<float> &out, int &w, int &h, std::string &why)
{
	const std::string p(path);
	const bool tif = ends_with(p, ".tif") || ends_with(p, ".tiff") || ends_with(p, ".TIF") || ends_with(p, ".TIFF");
	int c = 0, sample = 0;
	std::vector<float> in;
	const bool ok = ends_with(p, ".flo") ? read_flo(path, in, w, h, c)
	                : tif                ? read_tiff(path, in, w, h, c, &sample)
	                                     : read_pfm(path, in, w, h, c);
	if (!ok) {
		why = "could not read image";
		return false;
	}
	if (c == 1) {
		out.swap(in);
		return true;
	}
	// iio_hacky_uncolorize / _uncolorizea (lib/iio/iio.c:935-1006): 8-bit and
	// float samples with or without alpha, 16-bit without
	if (!(c == 3 || c == 4) || sample == 32 || (c == 4 && sample == 16)) {
		why = c == 3 || c == 4 ? "uncolorize type not supported" : "non-scalarizable image";
		return false;
	}
	const size_t wh = (size_t)w * h;
	out.resize(wh);
	for (size_t i = 0; i < wh; i++) {
		const double r = .299 * (double)in[i] + .587 * (double)in[wh + i] + .114 * (double)in[2 * wh + i];
		out[i] = sample == 8 ? (float)(uint8_t)r : sample == 16 ? (float)(uint16_t)r : (float)r;
	}
	return true;
}

bool write_flow(const char *path, const float *uv, int w, int h)
{
	const std::string p(path);
	if (ends_with(p, ".tif") || ends_with(p, ".tiff") || ends_with(p, ".TIF") || ends_with(p, ".TIFF"))
		return write_tiff(path, uv, w, h, 2);
	return write_flo(path, uv, w, h);
}

bool write_frame(const char *path, const float *planar, int w, int h, int c)
{
	const std::string p(path);
	if (ends_with(p, ".flo")) return c == 2 && write_flo(path, planar, w, h);
	if (ends_with(p, ".png")) return write_png(path, planar, w, h, c);
	if (ends_with(p, ".tif") || ends_with(p, ".tiff") || ends_with(p, ".TIF") || ends_with(p, ".TIFF"))
		return write_tiff(path, planar, w, h, c);
	return write_pfm(path, planar, w, h, c);
}

}  // namespace bm4dof_frames
