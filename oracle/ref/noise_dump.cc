// Test-oracle harness: the reference's noise tables and its procedural
// textures evaluated at given points, for the golden vectors of
// tests/golden/make_golden.py (textures group).  Only that script runs it.
//
// Input (text):
//   points N            then N lines "x y z" (texture-space points)
//   tables              the noise tables (NoiseGenerator::hash_, hashpntf_,
//                       BlenderNoiseGenerator::hashvectf_,
//                       StdPerlinNoiseGenerator::stdp_p_, stdp_g_)
//   noise TYPE          NoiseGenerator::newNoise(TYPE) at every point
//   turbulence TYPE OCT SIZE HARD   NoiseGenerator::turbulence
//   texture key=value ...           yafaray_createTexture with these
//                       parameters ("a,b,c,d" a colour, "a,b,c" a vector),
//                       then Texture::getColor and getFloat at every point
// Output (binary), per statement in order:
//   tables: u8 hash[512], f32 hashpntf[768], f32 hashvectf[768], u8 stdp_p[514], f32 stdp_g[514][3]
//   noise / turbulence: f32 [N]
//   texture: i32 status (0 created), f32 rgba[N][4], f32 value[N]
#include "yafaray_c_api.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#define private public
#define protected public
#include "noise/noise_generator.h"
#include "noise/generator/noise_blender.h"
#include "noise/generator/noise_perlin_standard.h"
#include "scene/scene.h"
#include "texture/texture.h"
#undef private
#undef protected

namespace {

void set_typed(yafaray_ParamMap *pm, const std::string &key, const std::string &val)
{
	double a, b, c, d;
	if(std::sscanf(val.c_str(), "%lf,%lf,%lf,%lf", &a, &b, &c, &d) == 4) { yafaray_setParamMapColor(pm, key.c_str(), a, b, c, d); return; }
	if(std::sscanf(val.c_str(), "%lf,%lf,%lf", &a, &b, &c) == 3) { yafaray_setParamMapVector(pm, key.c_str(), a, b, c); return; }
	if(val == "true" || val == "false") { yafaray_setParamMapBool(pm, key.c_str(), val == "true" ? YAFARAY_BOOL_TRUE : YAFARAY_BOOL_FALSE); return; }
	char *end = nullptr;
	const long iv = std::strtol(val.c_str(), &end, 10);
	if(end && *end == '\0') { yafaray_setParamMapInt(pm, key.c_str(), static_cast<int>(iv)); return; }
	const double dv = std::strtod(val.c_str(), &end);
	if(end && *end == '\0') { yafaray_setParamMapFloat(pm, key.c_str(), dv); return; }
	yafaray_setParamMapString(pm, key.c_str(), val.c_str());
}

yafaray::NoiseGenerator::NoiseType noise_type(const std::string &name)
{
	yafaray::NoiseGenerator::NoiseType t{yafaray::NoiseGenerator::NoiseType::PerlinImproved};
	for(const auto &[n, v] : yafaray::NoiseGenerator::NoiseType::map_)
		if(n == name) t = yafaray::NoiseGenerator::NoiseType{v.first};
	return t;
}

} // namespace

int main(int argc, char **argv)
{
	if(argc != 3) { std::fprintf(stderr, "usage: %s spec.txt out.bin\n", argv[0]); return 2; }
	std::ifstream in(argv[1]);
	if(!in) { std::perror("spec"); return 2; }
	FILE *out = std::fopen(argv[2], "wb");
	if(!out) { std::perror("out"); return 2; }
	yafaray_Logger *logger = yafaray_createLogger("oracle", nullptr, nullptr, YAFARAY_DISPLAY_CONSOLE_HIDDEN);
	yafaray_Scene *scene = yafaray_createScene(logger, "scene");
	std::vector<yafaray::Point3f> pts;
	std::string line;
	int n_tex = 0;
	while(std::getline(in, line))
	{
		std::istringstream ss(line);
		std::string kw;
		if(!(ss >> kw) || kw[0] == '#') continue;
		if(kw == "points")
		{
			size_t n = 0;
			ss >> n;
			pts.resize(n);
			for(size_t i = 0; i < n; ++i)
			{
				float x, y, z;
				in >> x >> y >> z;
				pts[i] = yafaray::Point3f{{x, y, z}};
			}
			std::getline(in, line);
		}
		else if(kw == "tables")
		{
			std::fwrite(yafaray::NoiseGenerator::hash_.data(), 1, 512, out);
			std::fwrite(yafaray::NoiseGenerator::hashpntf_.data(), 4, 768, out);
			std::fwrite(yafaray::BlenderNoiseGenerator::hashvectf_, 4, 768, out);
			std::fwrite(yafaray::StdPerlinNoiseGenerator::stdp_p_.data(), 1, 514, out);
			std::fwrite(yafaray::StdPerlinNoiseGenerator::stdp_g_, 4, 514 * 3, out);
		}
		else if(kw == "noise" || kw == "turbulence")
		{
			std::string type;
			ss >> type;
			const auto gen = yafaray::NoiseGenerator::newNoise(noise_type(type));
			int oct = 0; float size = 1.f; int hard = 0;
			if(kw == "turbulence") ss >> oct >> size >> hard;
			for(const auto &p : pts)
			{
				const float v = kw == "noise" ? (*gen)(p) : yafaray::NoiseGenerator::turbulence(gen.get(), p, oct, size, hard != 0);
				std::fwrite(&v, 4, 1, out);
			}
		}
		else if(kw == "texture")
		{
			yafaray_ParamMap *pm = yafaray_createParamMap();
			std::string kv;
			while(ss >> kv)
			{
				const size_t eq = kv.find('=');
				if(eq != std::string::npos) set_typed(pm, kv.substr(0, eq), kv.substr(eq + 1));
			}
			const std::string name = "tex" + std::to_string(n_tex++);
			const yafaray_ResultFlags rf = yafaray_createTexture(scene, name.c_str(), pm);
			yafaray_destroyParamMap(pm);
			const auto [tex, id, flags] = reinterpret_cast<yafaray::Scene *>(scene)->getTexture(name);
			const int status = (tex && !(rf & YAFARAY_RESULT_ERROR_WHILE_CREATING)) ? 0 : 1;
			std::fwrite(&status, 4, 1, out);
			for(const auto &p : pts)
			{
				const yafaray::Rgba c = tex ? tex->getColor(p) : yafaray::Rgba{0.f};
				const float v[4] = {c.r_, c.g_, c.b_, c.a_};
				std::fwrite(v, 4, 4, out);
			}
			for(const auto &p : pts)
			{
				const float v = tex ? tex->getFloat(p) : 0.f;
				std::fwrite(&v, 4, 1, out);
			}
		}
	}
	std::fclose(out);
	yafaray_destroyScene(scene);
	yafaray_destroyLogger(logger);
	return 0;
}
