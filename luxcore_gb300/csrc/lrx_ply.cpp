// PLY mesh ingestion: vertex positions and triangle indices from ascii,
// binary_little_endian and binary_big_endian PLY files, with the geometry
// semantics of the reference's loader (ExtTriangleMesh::LoadPly,
// src/luxrays/core/exttrianglemeshfile.cpp:207-290, over rply):
//   - element "vertex", properties x, y, z of any numeric type, stored as
//     float;
//   - element "face", list property "vertex_indices": a 3-index face is one
//     triangle, a 4-index face is split into (v0, v1, v2) and (v0, v2, v3),
//     faces of other lengths are dropped;
//   - a file with no vertices or no faces is an error.
// Other elements and properties are skipped.  Indices are not range-checked
// here (lrx_scene_create checks them), as in the reference.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "lrx_internal.h"

namespace {

enum class Fmt { Ascii, LittleEndian, BigEndian };
enum class Type { I8, U8, I16, U16, I32, U32, F32, F64, Bad };

Type parse_type(const std::string &t) {
	if (t == "char" || t == "int8") return Type::I8;
	if (t == "uchar" || t == "uint8") return Type::U8;
	if (t == "short" || t == "int16") return Type::I16;
	if (t == "ushort" || t == "uint16") return Type::U16;
	if (t == "int" || t == "int32") return Type::I32;
	if (t == "uint" || t == "uint32") return Type::U32;
	if (t == "float" || t == "float32") return Type::F32;
	if (t == "double" || t == "float64") return Type::F64;
	return Type::Bad;
}

size_t type_size(Type t) {
	switch (t) {
	case Type::I8: case Type::U8: return 1;
	case Type::I16: case Type::U16: return 2;
	case Type::I32: case Type::U32: case Type::F32: return 4;
	case Type::F64: return 8;
	default: return 0;
	}
}

struct Property {
	std::string name;
	Type type = Type::Bad;
	bool list = false;
	Type count_type = Type::Bad;
};

struct Element {
	std::string name;
	uint64_t count = 0;
	std::vector<Property> props;
};

// Sequential reader over the body of the file (after the header).
class Body {
public:
	Body(const std::vector<uint8_t> &data, size_t pos, Fmt fmt) : d(data), p(pos), fmt(fmt) {}

	bool value(Type t, double &out) {
		if (fmt == Fmt::Ascii) return ascii_value(out);
		const size_t n = type_size(t);
		if (n == 0 || p + n > d.size()) return false;
		uint8_t b[8];
		for (size_t k = 0; k < n; ++k) b[k] = d[p + (fmt == Fmt::BigEndian ? n - 1 - k : k)];
		p += n;
		switch (t) {
		case Type::I8: { int8_t v; std::memcpy(&v, b, 1); out = v; break; }
		case Type::U8: out = b[0]; break;
		case Type::I16: { int16_t v; std::memcpy(&v, b, 2); out = v; break; }
		case Type::U16: { uint16_t v; std::memcpy(&v, b, 2); out = v; break; }
		case Type::I32: { int32_t v; std::memcpy(&v, b, 4); out = v; break; }
		case Type::U32: { uint32_t v; std::memcpy(&v, b, 4); out = v; break; }
		case Type::F32: { float v; std::memcpy(&v, b, 4); out = v; break; }
		case Type::F64: { double v; std::memcpy(&v, b, 8); out = v; break; }
		default: return false;
		}
		return true;
	}

private:
	bool ascii_value(double &out) {
		while (p < d.size() && (d[p] == ' ' || d[p] == '\t' || d[p] == '\r' || d[p] == '\n')) ++p;
		if (p >= d.size()) return false;
		size_t e = p;
		while (e < d.size() && !(d[e] == ' ' || d[e] == '\t' || d[e] == '\r' || d[e] == '\n')) ++e;
		const std::string tok(reinterpret_cast<const char *>(d.data()) + p, e - p);
		p = e;
		char *end = nullptr;
		out = std::strtod(tok.c_str(), &end);
		return end && *end == '\0';
	}

	const std::vector<uint8_t> &d;
	size_t p;
	Fmt fmt;
};

lrx_status fail(const std::string &path, const std::string &why) {
	lrx::set_error("lrx_ply_load: '" + path + "': " + why);
	return LRX_ERR_INVALID_ARGUMENT;
}

}  // namespace

extern "C" lrx_status lrx_ply_load(const char *path, lrx_ply_mesh *out) {
	if (!path || !out) {
		lrx::set_error("lrx_ply_load: null argument");
		return LRX_ERR_INVALID_ARGUMENT;
	}
	std::memset(out, 0, sizeof(*out));
	const std::string name(path);
	std::vector<uint8_t> data;
	{
		std::unique_ptr<FILE, int (*)(FILE *)> f(std::fopen(path, "rb"), &std::fclose);
		if (!f) return fail(name, "unable to open");
		uint8_t buf[1 << 16];
		size_t n;
		while ((n = std::fread(buf, 1, sizeof(buf), f.get())) > 0) data.insert(data.end(), buf, buf + n);
	}
	// header: lines up to "end_header"
	size_t pos = 0;
	auto next_line = [&](std::string &line) -> bool {
		if (pos >= data.size()) return false;
		size_t e = pos;
		while (e < data.size() && data[e] != '\n') ++e;
		line.assign(reinterpret_cast<const char *>(data.data()) + pos, e - pos);
		if (!line.empty() && line.back() == '\r') line.pop_back();
		pos = e < data.size() ? e + 1 : e;
		return true;
	};
	std::string line;
	if (!next_line(line) || line != "ply") return fail(name, "not a PLY file");
	Fmt fmt = Fmt::Ascii;
	bool have_format = false, ended = false;
	std::vector<Element> elems;
	while (next_line(line)) {
		std::vector<std::string> w;
		{
			size_t i = 0;
			while (i < line.size()) {
				while (i < line.size() && (line[i] == ' ' || line[i] == '\t')) ++i;
				size_t j = i;
				while (j < line.size() && line[j] != ' ' && line[j] != '\t') ++j;
				if (j > i) w.push_back(line.substr(i, j - i));
				i = j;
			}
		}
		if (w.empty() || w[0] == "comment" || w[0] == "obj_info") continue;
		if (w[0] == "end_header") {
			ended = true;
			break;
		}
		if (w[0] == "format" && w.size() >= 2) {
			if (w[1] == "ascii") fmt = Fmt::Ascii;
			else if (w[1] == "binary_little_endian") fmt = Fmt::LittleEndian;
			else if (w[1] == "binary_big_endian") fmt = Fmt::BigEndian;
			else return fail(name, "unknown format " + w[1]);
			have_format = true;
		} else if (w[0] == "element" && w.size() >= 3) {
			Element e;
			e.name = w[1];
			char *end = nullptr;
			e.count = std::strtoull(w[2].c_str(), &end, 10);
			if (!end || *end) return fail(name, "bad element count");
			elems.push_back(e);
		} else if (w[0] == "property" && !elems.empty()) {
			Property pr;
			if (w.size() >= 5 && w[1] == "list") {
				pr.list = true;
				pr.count_type = parse_type(w[2]);
				pr.type = parse_type(w[3]);
				pr.name = w[4];
				if (pr.count_type == Type::Bad || pr.count_type == Type::F32 || pr.count_type == Type::F64)
					return fail(name, "bad list count type");
			} else if (w.size() >= 3) {
				pr.type = parse_type(w[1]);
				pr.name = w[2];
			} else {
				return fail(name, "bad property line");
			}
			if (pr.type == Type::Bad) return fail(name, "unknown property type");
			elems.back().props.push_back(pr);
		} else {
			return fail(name, "bad header line: " + line);
		}
	}
	if (!ended || !have_format) return fail(name, "unable to read PLY header");

	std::vector<float> verts;
	std::vector<uint32_t> tris;
	uint64_t n_verts = 0;
	bool have_faces = false;
	Body body(data, pos, fmt);
	for (const Element &e : elems) {
		const bool is_vertex = e.name == "vertex", is_face = e.name == "face";
		int ix = -1, iy = -1, iz = -1, ifc = -1;
		for (size_t k = 0; k < e.props.size(); ++k) {
			const Property &pr = e.props[k];
			if (is_vertex && !pr.list) {
				if (pr.name == "x") ix = (int)k;
				if (pr.name == "y") iy = (int)k;
				if (pr.name == "z") iz = (int)k;
			}
			if (is_face && pr.list && pr.name == "vertex_indices") ifc = (int)k;
		}
		const bool want_v = is_vertex && ix >= 0 && iy >= 0 && iz >= 0;
		if (want_v) {
			if (e.count > 0xffffffffull) return fail(name, "too many vertices");
			n_verts = e.count;
			verts.resize(3 * (size_t)e.count);
		}
		if (is_face && ifc >= 0) have_faces = true;
		for (uint64_t r = 0; r < e.count; ++r) {
			for (size_t k = 0; k < e.props.size(); ++k) {
				const Property &pr = e.props[k];
				if (!pr.list) {
					double v;
					if (!body.value(pr.type, v)) return fail(name, "unable to parse PLY file (truncated element " + e.name + ")");
					if (want_v) {
						if ((int)k == ix) verts[3 * r] = (float)v;
						else if ((int)k == iy) verts[3 * r + 1] = (float)v;
						else if ((int)k == iz) verts[3 * r + 2] = (float)v;
					}
					continue;
				}
				double cnt_d;
				if (!body.value(pr.count_type, cnt_d) || cnt_d < 0 || cnt_d > 1e6)
					return fail(name, "unable to parse PLY file (bad list length in " + e.name + ")");
				const uint32_t cnt = (uint32_t)cnt_d;
				uint32_t idx[4] = {0, 0, 0, 0};
				for (uint32_t j = 0; j < cnt; ++j) {
					double v;
					if (!body.value(pr.type, v)) return fail(name, "unable to parse PLY file (truncated list in " + e.name + ")");
					if (j < 4) idx[j] = (uint32_t)(int64_t)v;
				}
				if ((int)k == ifc) {
					if (cnt == 3) {
						tris.insert(tris.end(), {idx[0], idx[1], idx[2]});
					} else if (cnt == 4) {  // quad split as exttrianglemeshfile.cpp:221-233
						tris.insert(tris.end(), {idx[0], idx[1], idx[2], idx[0], idx[2], idx[3]});
					}
				}
			}
		}
	}
	if (n_verts == 0) return fail(name, "no vertices found");
	if (!have_faces || tris.empty()) return fail(name, "no faces found");
	if (tris.size() / 3 > 0xffffffffull) return fail(name, "too many triangles");
	out->vertices = static_cast<float *>(std::malloc(sizeof(float) * verts.size()));
	out->triangles = static_cast<uint32_t *>(std::malloc(sizeof(uint32_t) * tris.size()));
	if (!out->vertices || !out->triangles) {
		std::free(out->vertices);
		std::free(out->triangles);
		std::memset(out, 0, sizeof(*out));
		lrx::set_error("lrx_ply_load: out of host memory");
		return LRX_ERR_OUT_OF_MEMORY;
	}
	std::memcpy(out->vertices, verts.data(), sizeof(float) * verts.size());
	std::memcpy(out->triangles, tris.data(), sizeof(uint32_t) * tris.size());
	out->vertex_count = (uint32_t)n_verts;
	out->triangle_count = (uint32_t)(tris.size() / 3);
	return LRX_OK;
}

extern "C" void lrx_ply_free(lrx_ply_mesh *mesh) {
	if (!mesh) return;
	std::free(mesh->vertices);
	std::free(mesh->triangles);
	std::memset(mesh, 0, sizeof(*mesh));
}
