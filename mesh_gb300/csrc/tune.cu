// Autotuner registry: the launch variant chosen per (kernel, group,
// precision, lattice) key, measured once per process with CUDA events on the
// context's stream (kernels.cuh, Ops::choose_force). MESH_AUTOTUNE=0 in the
// environment disables timing and uses the default variants;
// MESH_FORCE_VARIANT=v pins momentum-step variant v where it is valid.
#include "field.cuh"

#include <cstdlib>
#include <map>
#include <mutex>

namespace meshgb {
namespace {
std::mutex g_mu;
std::map<std::string, std::pair<int, std::string>> &registry()
{
	static std::map<std::string, std::pair<int, std::string>> m;
	return m;
}
} // namespace

int tuned_variant(std::string const &key)
{
	std::lock_guard<std::mutex> lk(g_mu);
	auto it = registry().find(key);
	return it == registry().end() ? -1 : it->second.first;
}

void set_tuned_variant(std::string const &key, int variant, std::string const &report)
{
	std::lock_guard<std::mutex> lk(g_mu);
	registry()[key] = {variant, report};
}

namespace {
int g_force_override = -2; // -2: not yet read from MESH_FORCE_VARIANT
}
// the variant pinned by mesh_tune_force_variant, else by MESH_FORCE_VARIANT in
// the environment (read once), else -1 (autotune)
int force_override()
{
	if (g_force_override == -2)
	{
		char const *e = std::getenv("MESH_FORCE_VARIANT");
		g_force_override = e && *e ? std::atoi(e) : -1;
	}
	return g_force_override;
}
void set_force_override(int v) { g_force_override = v; }

bool autotune_enabled()
{
	char const *e = std::getenv("MESH_AUTOTUNE");
	return !(e && e[0] == '0');
}

std::string tune_report()
{
	std::lock_guard<std::mutex> lk(g_mu);
	std::string r;
	for (auto const &[k, v] : registry())
		r += k + ": " + v.second + "\n";
	return r;
}
} // namespace meshgb

extern "C" size_t mesh_tune_report(char *buf, size_t cap)
{
	std::string r = meshgb::tune_report();
	if (buf && cap)
	{
		size_t n = r.size() < cap - 1 ? r.size() : cap - 1;
		r.copy(buf, n);
		buf[n] = '\0';
	}
	return r.size() + 1;
}

extern "C" int mesh_tune_force_variant(int variant)
{
	if (variant < -1 || variant >= 64)
		return MESH_ERR_ARG;
	meshgb::set_force_override(variant);
	return MESH_OK;
}
