// Gauge-configuration files. The reference's writer stores a LatticeStack as
// one dataset of shape [Nd, X, Y, Z, T, ncomp] with the grid and the group
// as attributes, and readConfig checks both on load (writeToFile /
// readFromFile, src/lattice/lattice.h:205-252; readConfig,
// src/gauge/utils.h:188-219; both are commented out or assert in the
// reference, and HDF5 is not part of this build). Here the same dataset, in
// the reference's host layout (component-major, sites lexicographic with
// dimension 0 slowest, objects as full group-type reals), follows a 72-byte
// little-endian header:
//   char     magic[8]   "MESHCFG1"
//   int32    version    1
//   int32    group, precision (1 float, 2 double), kind (0 group, 1 algebra)
//   int32    nd, nstack, dims[4] (unused entries 0)
//   uint64   trajectory (HMC trajectories done; 0 for a plain field)
//   uint64   seed       (HMC stream key; 0 for a plain field)
//   uint64   checksum   sum of the data as little-endian uint64 words mod
//                       2^64 (a zero-padded tail word)
#include "field.cuh"

#include <cstdio>
#include <cstring>
#include <memory>
#include <string>

namespace meshgb {

static_assert(sizeof(ConfigHeader) == 72, "configuration header layout");

namespace {

struct FileCloser
{
	void operator()(std::FILE *f) const
	{
		if (f)
			std::fclose(f);
	}
};
using File = std::unique_ptr<std::FILE, FileCloser>;

uint64_t checksum(void const *data, size_t bytes)
{
	auto const *p = static_cast<unsigned char const *>(data);
	uint64_t s = 0;
	size_t n = bytes / 8;
	for (size_t i = 0; i < n; ++i)
	{
		uint64_t w;
		std::memcpy(&w, p + 8 * i, 8);
		s += w;
	}
	if (bytes % 8)
	{
		uint64_t w = 0;
		std::memcpy(&w, p + 8 * n, bytes % 8);
		s += w;
	}
	return s;
}

File open_file(char const *path, char const *mode)
{
	require(path != nullptr && path[0] != '\0', "empty path");
	File f(std::fopen(path, mode));
	if (!f)
		throw Error(MESH_ERR_ARG, std::string("cannot open configuration file '") + path + "'");
	return f;
}

} // namespace

size_t config_data_bytes(ConfigHeader const &h)
{
	size_t V = 1;
	for (int i = 0; i < h.nd; ++i)
		V *= size_t(h.dims[i]);
	return size_t(h.nstack) * V * size_t(group_nr(h.group)) * (h.precision == MESH_F32 ? 4 : 8);
}

ConfigHeader config_header_of(Field const &f, uint64_t trajectory, uint64_t seed)
{
	ConfigHeader h{};
	std::memcpy(h.magic, "MESHCFG1", 8);
	h.version = 1;
	h.group = f.group;
	h.precision = f.prec;
	h.kind = f.kind;
	h.nd = f.nd;
	h.nstack = f.nstack;
	for (int i = 0; i < 4; ++i)
		h.dims[i] = i < f.nd ? f.dims[i] : 0;
	h.trajectory = trajectory;
	h.seed = seed;
	return h;
}

void config_write(char const *path, ConfigHeader h, void const *data, size_t bytes)
{
	require(bytes == config_data_bytes(h), "data size does not match the configuration header");
	h.checksum = checksum(data, bytes);
	File f = open_file(path, "wb");
	bool ok = std::fwrite(&h, sizeof(h), 1, f.get()) == 1 && std::fwrite(data, 1, bytes, f.get()) == bytes;
	ok = (std::fflush(f.get()) == 0) && ok;
	if (!ok)
		throw Error(MESH_ERR_ARG, std::string("write failed: '") + path + "'");
}

ConfigHeader config_read_header(char const *path)
{
	File f = open_file(path, "rb");
	ConfigHeader h{};
	if (std::fread(&h, sizeof(h), 1, f.get()) != 1 || std::memcmp(h.magic, "MESHCFG1", 8) != 0)
		throw Error(MESH_ERR_ARG, std::string("not a configuration file: '") + path + "'");
	require(h.version == 1, "unsupported configuration file version");
	require(h.group >= 1 && h.group <= 3 && (h.precision == MESH_F32 || h.precision == MESH_F64) &&
	            (h.kind == MESH_GROUP || h.kind == MESH_ALGEBRA) && h.nd >= 2 && h.nd <= 4 && h.nstack >= 1 &&
	            h.nstack <= 64,
	        "corrupt configuration header");
	for (int i = 0; i < h.nd; ++i)
		require(h.dims[i] >= 2 && h.dims[i] < 256 && h.dims[i] % 2 == 0, "corrupt configuration header (extents)");
	return h;
}

void config_read_data(char const *path, ConfigHeader const &h, void *data, size_t bytes)
{
	require(bytes == config_data_bytes(h), "buffer size does not match the configuration file");
	File f = open_file(path, "rb");
	ConfigHeader skip;
	if (std::fread(&skip, sizeof(skip), 1, f.get()) != 1 || std::fread(data, 1, bytes, f.get()) != bytes)
		throw Error(MESH_ERR_ARG, std::string("configuration file truncated: '") + path + "'");
	if (checksum(data, bytes) != h.checksum)
		throw Error(MESH_ERR_STATE, std::string("configuration file checksum mismatch: '") + path + "'");
}

// refuses a file whose group, precision, kind or grid differ from the field
// (the checks of readConfig, utils.h:198-208)
void config_check_matches(ConfigHeader const &h, Field const &f)
{
	if (h.group != f.group || h.kind != f.kind)
		throw Error(MESH_ERR_STATE, "group mismatch on load");
	if (h.precision != f.prec)
		throw Error(MESH_ERR_STATE, "precision mismatch on load");
	bool same = h.nd == f.nd && h.nstack == f.nstack;
	for (int i = 0; same && i < f.nd; ++i)
		same = h.dims[i] == f.dims[i];
	if (!same)
		throw Error(MESH_ERR_STATE, "grid mismatch on load");
}

} // namespace meshgb
