// vtk_serializer.cpp -- see vtk_serializer.h.
#include "vtk_serializer.h"

#include <bit>
#include <cstdint>
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <stdexcept>

#include "gb300_solver.h"
#include "microenvironment.h"

static_assert(std::endian::native == std::endian::little, "the writer emits little-endian arrays");

namespace physicore::biofvm {

namespace {

std::string xml_escape(const std::string& s)
{
	std::string out;
	for (char c : s)
		switch (c)
		{
		case '<': out += "&lt;"; break;
		case '>': out += "&gt;"; break;
		case '&': out += "&amp;"; break;
		case '"': out += "&quot;"; break;
		default: out += c;
		}
	return out;
}

} // namespace

vtk_serializer::vtk_serializer(std::string_view output_dir, const microenvironment& m)
	: output_dir_(output_dir), vtks_dir_((std::filesystem::path(output_dir) / "vtk_microenvironment").string()),
	  pvd_contents_("<?xml version=\"1.0\"?>\n<VTKFile type=\"Collection\" version=\"0.1\" "
					"byte_order=\"LittleEndian\">\n  <Collection>\n")
{
	std::filesystem::create_directories(vtks_dir_);
	const cartesian_mesh& g = m.mesh;
	for (int a = 0; a < 3; a++)
	{
		const bool used = a < 2 || g.dims == 3;
		const long long start = used ? (long long)(g.bounding_box_mins[a] / (sindex_t)g.voxel_shape[a]) : 0;
		extent_[2 * a] = start;
		extent_[2 * a + 1] = used ? start + (long long)g.grid_shape[a] : 0;
		spacing_[a] = used ? (double)g.voxel_shape[a] : 0.0;
	}
	std::ostringstream ext;
	for (int i = 0; i < 6; i++)
		ext << (i ? " " : "") << extent_[i];
	std::ostringstream h;
	h.precision(17);
	h << "<?xml version=\"1.0\"?>\n"
	  << "<VTKFile type=\"ImageData\" version=\"1.0\" byte_order=\"LittleEndian\" header_type=\"UInt64\">\n"
	  << "  <ImageData WholeExtent=\"" << ext.str() << "\" Origin=\"0 0 0\" Spacing=\"" << spacing_[0] << " "
	  << spacing_[1] << " " << spacing_[2] << "\" Direction=\"1 0 0 0 1 0 0 0 1\">\n"
	  << "    <Piece Extent=\"" << ext.str() << "\">\n"
	  << "      <PointData>\n      </PointData>\n      <CellData>\n";
	const std::uint64_t V = g.voxel_count();
	for (index_t s = 0; s < m.substrates_count; s++)
	{
		const std::string name = s < m.substrates_names.size() ? m.substrates_names[s] : "density_" + std::to_string(s);
		h << "        <DataArray type=\"Float64\" Name=\"" << xml_escape(name)
		  << "\" format=\"appended\" RangeMin=\"0\" RangeMax=\"0\" offset=\"" << s * (8 + V * 8) << "\"/>\n";
	}
	h << "      </CellData>\n    </Piece>\n  </ImageData>\n  <AppendedData encoding=\"raw\">\n   _";
	header_ = h.str();
}

void vtk_serializer::serialize(const microenvironment& m, real_t current_time)
{
	const cartesian_mesh& g = m.mesh;
	const std::uint64_t V = g.voxel_count(), S = m.substrates_count;
	planar_.resize(V * S);
	using kernels::gb300_solver::gb300_solver;
	const auto* gpu = dynamic_cast<const gb300_solver*>(m.solver.get());
	if (gpu && gpu->context())
		gpu->read_field_planar(planar_.data());
	else
		for (index_t s = 0; s < S; s++)
			for (index_t z = 0; z < g.grid_shape[2]; z++)
				for (index_t y = 0; y < g.grid_shape[1]; y++)
					for (index_t x = 0; x < g.grid_shape[0]; x++)
						planar_[s * V + g.linearize(x, y, z)] = m.get_substrate_density(s, x, y, z);

	char name[64];
	std::snprintf(name, sizeof name, "microenvironment_%06zu.vti", iteration_);
	const std::filesystem::path path = std::filesystem::path(vtks_dir_) / name;
	{
		std::ofstream f(path, std::ios::binary | std::ios::trunc);
		if (!f)
			throw std::runtime_error("vtk_serializer: cannot write " + path.string());
		f.write(header_.data(), (std::streamsize)header_.size());
		const std::uint64_t bytes = V * sizeof(real_t);
		for (std::uint64_t s = 0; s < S; s++)
		{
			f.write(reinterpret_cast<const char*>(&bytes), sizeof bytes);
			f.write(reinterpret_cast<const char*>(planar_.data() + s * V), (std::streamsize)bytes);
		}
		const char tail[] = "\n  </AppendedData>\n</VTKFile>\n";
		f.write(tail, sizeof tail - 1);
		if (!f)
			throw std::runtime_error("vtk_serializer: write to " + path.string() + " failed");
	}
	last_file_ = path.string();
	append_to_pvd(name, current_time);
	iteration_++;
}

void vtk_serializer::append_to_pvd(const std::string& file_name, real_t current_time)
{
	const std::filesystem::path file = std::filesystem::path(vtks_dir_) / file_name;
	pvd_contents_ += "    <DataSet timestep=\"" + std::to_string(current_time) + "\" group=\"\" part=\"0\" file=\"" +
					 std::filesystem::relative(file, output_dir_).string() + "\" />\n";
	std::ofstream pvd(std::filesystem::path(output_dir_) / "microenvironment.pvd", std::ios::trunc);
	pvd << pvd_contents_ << "  </Collection>\n</VTKFile>";
}

} // namespace physicore::biofvm
