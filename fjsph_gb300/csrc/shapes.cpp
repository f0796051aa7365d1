/*
 * shapes.cpp -- initial particles from the reference's block files.
 *
 * Restates, on the host, what src/Init.cpp:61-496 (Check_Intersection, Generate_Points,
 * Init_Particles), src/shapes/shapes.cpp:400-600 (read_shapes_bmap with the IOFunctions.h
 * Get_* rules) and the shape classes of src/shapes/ (line, square, circle, arc, cylinder,
 * inlet, coordinates; check_input and generate_points, 2D and 3D) do before the first step:
 *
 *   read blocks  ->  check_input per block  ->  generate_points  ->  intersection culling
 *   ->  state in reference index order (boundary blocks, then fluid blocks), LIMITS entries,
 *   inlet back/buffer tables, hydrostatic pressure.
 *
 * The result goes to the device through the usual upload; nothing here touches the GPU.  The
 * reference's quirks are kept where they change the particle set (each one is commented), and
 * its exit(-1) paths become FJSPH_E_ARG with the message in the log.  Each generator starts a
 * default-constructed std::default_random_engine and draws uniform(0, eps * dx) perturbations,
 * as upstream; where upstream passes two draws as constructor arguments (evaluation order
 * unspecified in C++) they are drawn left to right here.
 */
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/fjsph_gb300.h"

namespace {

constexpr double kDefault = 9999999.0;               /* default_val, src/VarDefs.h:195 */
constexpr double kEps = 2.220446049250313080847e-16; /* MEPSILON for double */
constexpr double kPi = 3.14159265358979323846;
const char *const kWhitespace = " \n\r\t\f\v";

enum ShapeType { linePlane = 0, squareCube, circleSphere, cylinder, arcSection, coordDef, inletZone, hollow, solid };
enum BoundSolver { DBC = 0, pressure_G, ghost };

using V = std::array<double, 3>;
struct M3 {
    double a[3][3];
};

inline V vadd(const V &x, const V &y) { return {x[0] + y[0], x[1] + y[1], x[2] + y[2]}; }
inline V vsub(const V &x, const V &y) { return {x[0] - y[0], x[1] - y[1], x[2] - y[2]}; }
inline V vmul(const V &x, double s) { return {x[0] * s, x[1] * s, x[2] * s}; }
inline V vdiv(const V &x, double s) { return {x[0] / s, x[1] / s, x[2] / s}; }
inline double vdot(const V &x, const V &y) { return x[0] * y[0] + x[1] * y[1] + x[2] * y[2]; }
inline double vsq(const V &x) { return vdot(x, x); }
inline double vnorm(const V &x) { return std::sqrt(vsq(x)); }
inline V vcross(const V &x, const V &y) {
    return {x[1] * y[2] - x[2] * y[1], x[2] * y[0] - x[0] * y[2], x[0] * y[1] - x[1] * y[0]};
}
/* Eigen's normalized(): divide by the norm; a zero vector stays zero */
inline V vnormalized(const V &x) {
    const double n = vsq(x);
    return n > 0.0 ? vdiv(x, std::sqrt(n)) : x;
}
inline M3 identity() {
    M3 m{};
    for (int i = 0; i < 3; ++i) m.a[i][i] = 1.0;
    return m;
}
inline V mv(const M3 &m, const V &x) {
    V r;
    for (int i = 0; i < 3; ++i) r[i] = m.a[i][0] * x[0] + m.a[i][1] * x[1] + m.a[i][2] * x[2];
    return r;
}
inline bool is_identity(const M3 &m, int D) {
    for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j)
            if (m.a[i][j] != (i == j ? 1.0 : 0.0)) return false;
    return true;
}

/* GetRotationMat (src/Geometry.h:14-43), angles in radians.  3D: the rotation of the quaternion
 * product AngleAxis(a0, x) * AngleAxis(-a1, y) * AngleAxis(a2, z). */
M3 rotation(const V &ang, int D) {
    M3 m = identity();
    if (D == 2) {
        const double c = std::cos(ang[0]), s = std::sin(ang[0]);
        m.a[0][0] = c; m.a[0][1] = -s;
        m.a[1][0] = s; m.a[1][1] = c;
        return m;
    }
    struct Q { double w, x, y, z; };
    auto axis = [](double angle, int k) {
        const double h = 0.5 * angle;
        Q q{std::cos(h), 0.0, 0.0, 0.0};
        const double s = std::sin(h);
        (k == 0 ? q.x : k == 1 ? q.y : q.z) = s;
        return q;
    };
    auto mul = [](const Q &a, const Q &b) {
        return Q{a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z, a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y,
                 a.w * b.y + a.y * b.w + a.z * b.x - a.x * b.z, a.w * b.z + a.z * b.w + a.x * b.y - a.y * b.x};
    };
    const Q q = mul(mul(axis(ang[0], 0), axis(-ang[1], 1)), axis(ang[2], 2));
    const double tx = 2 * q.x, ty = 2 * q.y, tz = 2 * q.z;
    const double twx = tx * q.w, twy = ty * q.w, twz = tz * q.w;
    const double txx = tx * q.x, txy = ty * q.x, txz = tz * q.x;
    const double tyy = ty * q.y, tyz = tz * q.y, tzz = tz * q.z;
    m.a[0][0] = 1 - (tyy + tzz); m.a[0][1] = txy - twz;       m.a[0][2] = txz + twy;
    m.a[1][0] = txy + twz;       m.a[1][1] = 1 - (txx + tzz); m.a[1][2] = tyz - twx;
    m.a[2][0] = txz - twy;       m.a[2][1] = tyz + twx;       m.a[2][2] = 1 - (txx + tyy);
    return m;
}

/* ---- IOFunctions.h Get_* rules ------------------------------------------------------------ */

std::string ltrim(const std::string &s) {
    const size_t a = s.find_first_not_of(kWhitespace);
    return a == std::string::npos ? "" : s.substr(a);
}
std::string rtrim(const std::string &s) {
    const size_t b = s.find_last_not_of(kWhitespace);
    return b == std::string::npos ? "" : s.substr(0, b + 1);
}
/* Get_Parameter_Value: text after the first ':' (lines reach here with comments removed) */
std::string param_value(const std::string &line) { return ltrim(rtrim(line.substr(line.find(':') + 1))); }
/* the key matches when the text before the first ':' equals it after a left trim */
bool key_is(const std::string &line, const char *key) {
    const size_t pos = line.find(':');
    return pos != std::string::npos && ltrim(line.substr(0, pos)) == key;
}
/* istream >> double / int / bool: a failed extraction stores 0 */
double parse_double(const std::string &t) {
    std::istringstream is(t);
    double v = 0.0;
    if (!(is >> v)) return 0.0;
    return v;
}
long parse_long(const std::string &t) {
    std::istringstream is(t);
    long v = 0;
    if (!(is >> v)) return 0;
    return v;
}
bool parse_bool(const std::string &t) { /* 0 -> false, 1 -> true, other numbers -> true */
    std::istringstream is(t);
    long v = 0;
    if (!(is >> v)) return false;
    return v != 0;
}
void get_string(const std::string &line, const char *key, std::string &out) {
    if (key_is(line, key)) out = param_value(line);
}
void get_double(const std::string &line, const char *key, double &out) {
    if (key_is(line, key)) out = parse_double(param_value(line));
}
void get_int(const std::string &line, const char *key, int &out) {
    if (key_is(line, key)) out = (int)parse_long(param_value(line));
}
void get_bool(const std::string &line, const char *key, bool &out) {
    if (key_is(line, key)) out = parse_bool(param_value(line));
}
/* Get_Vector: `dim` comma-separated components; missing ones read as 0 */
void get_vector(const std::string &line, const char *key, V &out, int D) {
    if (!key_is(line, key)) return;
    std::istringstream is(param_value(line));
    for (int k = 0; k < D; ++k) {
        std::string tok;
        std::getline(is, tok, ',');
        out[k] = parse_double(tok);
    }
}

/* ---- blocks --------------------------------------------------------------------------------- */

struct Block { /* ShapeBlock, src/shapes/shapes.h:11-103 */
    bool write_data = false, no_slip = false, particle_order = false;
    std::string name, shape, subshape, filename, position_filename, solver_name, particle_order_str,
        inlet_bc_type;
    int bound_type = -1, sub_bound_type = -1, fixed_vel_or_dynamic = 0, bound_solver = pressure_G;
    int ni = 0, nj = 0, nk = 0;
    int64_t npts = 0, ntimes = 0;
    double insconst = kDefault, delconst = kDefault, aeroconst = kDefault;
    double dx = -1, radius = -1, arc_start = -1, arc_end = -1, arclength = kDefault, thickness = -1,
           length = -1, sstraight = 0, estraight = 0;
    double vmag = 0, press = 0, dens = 1000, nu = -1;
    V insert_norm{1, 0, 0}, delete_norm{1, 0, 0}, aero_norm{1, 0, 0}, normal{1, 0, 0}, angles{0, 0, 0};
    M3 rotmat = identity();
    V start, end, right, mid, centre, vel{0, 0, 0};
    std::vector<int64_t> back;
    std::vector<std::vector<int64_t>> buffer;
    std::vector<int> bc, intersect;
    std::vector<double> times;
    std::vector<V> pos, vels, coords;
    int64_t estimated = 0, generated = 0, kept = 0;

    explicit Block(int D) {
        const double z = D == 3 ? kDefault : 0.0;
        start = end = right = mid = centre = V{kDefault, kDefault, z};
    }
};

struct Geometry {
    fjsph_settings s{};
    int D = 2;
    double gs_running = 0; /* the globalspacing every check_input raises (check_input_post) */
    std::vector<Block> bound, fluid;
    std::string log;
    bool built = false;
    /* assembled */
    std::vector<V> xi, v;
    std::vector<double> rho, p, m;
    std::vector<int32_t> b;
    std::vector<fjsph_block> limits;
    struct Inlet {
        int32_t block;
        std::vector<int64_t> back;
        std::vector<std::vector<int64_t>> buffer;
    };
    std::vector<Inlet> inlets;
    int64_t n_bound_points = 0;

    void msg(const char *fmt, ...) __attribute__((format(printf, 2, 3)));
    bool check_vector(const V &x) const {
        for (int k = 0; k < D; ++k)
            if (x[k] == kDefault) return false;
        return true;
    }
    bool is_unit_x(const V &x) const {
        for (int k = 0; k < D; ++k)
            if (x[k] != (k == 0 ? 1.0 : 0.0)) return false;
        return true;
    }
    double norm_d(const V &x) const { return vnorm(x); }
};

void Geometry::msg(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    log += buf;
    log += '\n';
}

/* create_shape (src/shapes/shapes.cpp:166-228): 2D names Line/Square/Circle/Arc, 3D names
 * Plane/Cube/Sphere/Arch; Cylinder, Inlet and Coordinates in both */
bool make_block(Geometry &g, const std::string &shape, Block &out) {
    out = Block(g.D);
    const bool two = g.D == 2;
    if (shape == (two ? "Line" : "Plane")) out.bound_type = linePlane;
    else if (shape == (two ? "Square" : "Cube")) out.bound_type = squareCube;
    else if (shape == (two ? "Circle" : "Sphere")) out.bound_type = circleSphere;
    else if (shape == (two ? "Arc" : "Arch")) out.bound_type = arcSection;
    else if (shape == "Cylinder") out.bound_type = cylinder;
    else if (shape == "Inlet") out.bound_type = inletZone;
    else if (shape == "Coordinates") out.bound_type = coordDef;
    else {
        g.msg("block shape \"%s\" is not a known shape", shape.c_str());
        return false;
    }
    return true;
}

/* read_shapes_bmap (src/shapes/shapes.cpp:400-600) on the file's text */
int read_bmap(Geometry &g, const std::string &text, std::vector<Block> &blocks) {
    int fault = 0;
    std::vector<Block> shapes;
    {
        std::istringstream in(text);
        std::string line, shape_name;
        while (std::getline(in, line)) {
            const size_t c = line.find_first_of('#');
            if (c != std::string::npos) line = line.substr(0, c + 1); /* first pass keeps the '#' */
            get_string(line, "Shape", shape_name);
            if (line.find("block end") != std::string::npos) {
                Block nb(g.D);
                if (!make_block(g, shape_name, nb)) fault = 1;
                shapes.push_back(std::move(nb));
                shape_name.clear();
            }
        }
    }
    const size_t nblocks = shapes.size();
    if (nblocks) {
        std::istringstream in(text);
        std::string line;
        size_t block = 0;
        while (std::getline(in, line)) {
            const size_t c = line.find_first_of('#');
            if (c != std::string::npos) line = line.substr(0, c);
            Block &b = shapes[block];
            const int D = g.D;
            get_string(line, "Name", b.name);
            get_string(line, "Shape", b.shape);
            get_string(line, "Sub-shape", b.subshape);
            get_string(line, "Boundary solver", b.solver_name);
            get_bool(line, "Write surface data (0/1)", b.write_data);
            get_int(line, "Fixed velocity or dynamic inlet BC (0/1)", b.fixed_vel_or_dynamic);
            /* the JSON reader's string form ("Fixed Velocity" / "Dynamic"), src/shapes/shapes.cpp:286 */
            get_string(line, "Fixed velocity or dynamic inlet BC", b.inlet_bc_type);
            get_vector(line, "Aerodynamic entry normal", b.aero_norm, D);
            get_vector(line, "Deletion normal", b.delete_norm, D);
            get_vector(line, "Insertion normal", b.insert_norm, D);
            get_double(line, "Aerodynamic entry plane constant", b.aeroconst);
            get_double(line, "Deletion plane constant", b.delconst);
            get_double(line, "Insertion plane constant", b.insconst);
            get_double(line, "Pipe depth", b.thickness);
            get_int(line, "i-direction count", b.ni);
            get_int(line, "j-direction count", b.nj);
            get_int(line, "k-direction count", b.nk);
            get_vector(line, "Normal vector", b.normal, D);
            get_vector(line, "Rotation angles", b.angles, D);
            get_double(line, "Rotation angle", b.angles[0]);
            get_vector(line, "Start coordinate", b.start, D);
            get_vector(line, "End coordinate", b.end, D);
            get_vector(line, "Right coordinate", b.right, D);
            get_vector(line, "Midpoint coordinate", b.mid, D);
            get_vector(line, "Centre coordinate", b.centre, D);
            get_vector(line, "Arch normal", b.right, D);
            get_double(line, "Radius", b.radius);
            get_double(line, "Length", b.length);
            get_double(line, "Arc start (degree)", b.arc_start);
            get_double(line, "Arc end (degree)", b.arc_end);
            get_double(line, "Arc length (degree)", b.arclength);
            get_double(line, "Starting straight length", b.sstraight);
            get_double(line, "Ending straight length", b.estraight);
            get_double(line, "Particle spacing", b.dx);
            get_bool(line, "Particle ordering (0=grid,1=HCP)", b.particle_order);
            get_double(line, "Wall thickness", b.thickness);
            get_int(line, "Wall radial particle count", b.nk);
            get_bool(line, "Wall is no slip (0/1)", b.no_slip);
            get_string(line, "Coordinate filename", b.filename);
            get_vector(line, "Starting velocity", b.vel, D);
            get_double(line, "Starting jet velocity", b.vmag);
            get_double(line, "Starting pressure", b.press);
            get_double(line, "Starting density", b.dens);
            get_string(line, "Time data filename", b.position_filename);

            if (line.find("Coordinate data:") != std::string::npos) {
                /* the line after the key is skipped; then the count and the coordinates */
                std::string skip;
                std::getline(in, skip);
                long n = 0;
                in >> n;
                if (n < 0 || !in) n = 0;
                b.npts = n;
                b.coords.assign((size_t)n, V{0, 0, 0});
                for (long i = 0; i < n; ++i)
                    for (int k = 0; k < D; ++k) in >> b.coords[(size_t)i][k];
            }
            const bool tpos = line.find("Time position data") != std::string::npos;
            const bool tvel = line.find("Time velocity data") != std::string::npos;
            if (tpos || tvel) {
                std::string tmp;
                std::getline(in, tmp);
                long nt = parse_long(tmp);
                if (nt < 0) nt = 0;
                b.ntimes = nt;
                b.times.assign((size_t)nt, 0.0);
                std::vector<V> &dst = tpos ? b.pos : b.vels;
                dst.assign((size_t)nt, V{0, 0, 0});
                for (long i = 0; i < nt; ++i) {
                    std::getline(in, tmp);
                    std::istringstream row(tmp);
                    row >> b.times[(size_t)i];
                    for (int k = 0; k < D; ++k) row >> dst[(size_t)i][k];
                }
            }
            if (line.find("block end") != std::string::npos) {
                if (++block == nblocks) break;
            }
        }
    }
    blocks.insert(blocks.end(), std::make_move_iterator(shapes.begin()), std::make_move_iterator(shapes.end()));
    return fault;
}

/* ---- check_input ------------------------------------------------------------------------------ */

void check_base(Geometry &g, Block &b, int &fault) { /* ShapeBlock::check_input, shapes.cpp:21-160 */
    const fjsph_settings &s = g.s;
    if (s.scale != 1.0) {
        for (V *x : {&b.start, &b.end, &b.right, &b.mid, &b.centre})
            if (g.check_vector(*x)) *x = vmul(*x, s.scale);
        if (b.aeroconst != kDefault) b.aeroconst *= s.scale;
        if (b.insconst != kDefault) b.insconst *= s.scale;
        if (b.delconst != kDefault) b.delconst *= s.scale;
    }
    if (!b.position_filename.empty() && b.ntimes != 0) {
        if (b.times.empty()) {
            g.msg("block \"%s\": motion values without times", b.name.c_str());
            fault = 1;
        }
        if (b.pos.empty() && b.vels.empty()) {
            g.msg("block \"%s\": motion table lengths differ", b.name.c_str());
            fault = 1;
        }
    }
    if (b.bound_type == -1) {
        g.msg("block \"%s\": no shape given", b.name.c_str());
        fault = 1;
    }
    if (!b.solver_name.empty()) {
        if (b.solver_name == "DBC") b.bound_solver = DBC;
        else if (b.solver_name == "Pressure-Gradient") b.bound_solver = pressure_G;
        else if (b.solver_name == "Ghost") b.bound_solver = ghost;
        else g.msg("note: unknown boundary solver; the Pressure-Gradient solver is used");
    }
    if (!b.inlet_bc_type.empty()) {
        if (b.inlet_bc_type == "Fixed Velocity") b.fixed_vel_or_dynamic = 0;
        else if (b.inlet_bc_type == "Dynamic") b.fixed_vel_or_dynamic = 1;
        else g.msg("note: unknown inlet velocity type; a fixed inlet velocity is used");
    }
    if (!b.particle_order_str.empty()) {
        if (b.particle_order_str == "Grid") b.particle_order = false;
        else if (b.particle_order_str == "HCP") b.particle_order = true;
        else g.msg("note: unknown packing type; grid packing is used");
    }
    if (b.press != 0) {
        /* upstream raises to gam here, not 1/gam (get_density uses 1/gam) */
        const double B = s.rho_rest * (s.speed_sound * s.speed_sound) / s.gam;
        b.dens = std::pow(((b.press - s.press_pipe) / B + 1.0), s.gam) * s.rho_rest;
    } else {
        b.dens = s.rho_rest;
    }
    if (b.nu < 0) b.nu = s.nu;
}

void check_post(Geometry &g, Block &b) {
    g.gs_running = std::max(b.dx, g.gs_running);
    b.npts = b.npts > 1 ? b.npts : 1;
    b.estimated = b.npts;
}

int iceil(double x) { return static_cast<int>(std::ceil(x)); }

void check_line(Geometry &g, Block &b, int &fault) { /* src/shapes/line.cpp:8-125 */
    const double gs = g.gs_running;
    const int D = g.D;
    if (!g.check_vector(b.start)) { g.msg("block \"%s\": start point missing", b.name.c_str()); fault = 1; }
    if (!g.check_vector(b.end)) { g.msg("block \"%s\": end point missing", b.name.c_str()); fault = 1; }
    if (D == 3 && !g.check_vector(b.right)) { g.msg("block \"%s\": end point missing", b.name.c_str()); fault = 1; }
    if (b.dx < 0 && (b.ni < 0 || (D == 3 && b.nj < 0))) b.dx = gs;
    if (D == 2) {
        if (b.ni > 0 && b.dx < 0) b.dx = vnorm(vsub(b.end, b.start)) / double(b.ni);
    } else if (b.ni > 0 && b.nj > 0) {
        b.dx = std::min(vnorm(vsub(b.right, b.start)) / double(b.ni), vnorm(vsub(b.end, b.right)) / double(b.nj));
    }
    if (b.thickness < 0) {
        if (b.nk < 0) { g.msg("block \"%s\": wall thickness or layer count missing", b.name.c_str()); fault = 1; }
    } else if (b.nk < 0) { /* the thickness is used only with a negative count */
        b.nk = b.particle_order ? iceil(b.thickness / b.dx / std::sqrt(3.0) * 2.0) : iceil(b.thickness / b.dx);
    }
    b.nk = b.nk > 1 ? b.nk : 1;
    if (b.ni > 0) {
        if (D == 2) b.npts = (int64_t)b.ni * b.nk;
        else {
            if (b.nj < 1) {
                g.msg("note: an i count is given without a j count");
                b.nj = std::max(iceil(vnorm(vsub(b.end, b.right)) / gs), 1);
            }
            b.npts = (int64_t)b.ni * b.nj * b.nk;
        }
    } else if (D == 2) {
        b.ni = std::max(iceil(vnorm(vsub(b.end, b.start)) / gs), 1);
        b.npts = (int64_t)b.ni * b.nk;
    } else {
        b.ni = iceil(vnorm(vsub(b.right, b.start)) / gs);
        b.nj = b.particle_order ? iceil(vnorm(vsub(b.end, b.right)) / gs / std::sqrt(3.0) * 2.0)
                                : iceil(vnorm(vsub(b.end, b.right)) / gs);
        b.ni = std::max(b.ni, 1);
        b.nj = std::max(b.nj, 1);
        b.npts = (int64_t)b.ni * b.nj * b.nk;
    }
}

/* lattice counts of a box from start to end (square.cpp:62-90, circle.cpp:44-72) */
void box_counts(const Block &b, double gs, int D, int &ni, int &nj, int &nk) {
    if (b.particle_order) {
        ni = iceil((b.end[0] - b.start[0]) / gs);
        nj = iceil((b.end[1] - b.start[1]) / gs / std::sqrt(3.0) * 2.0);
        nk = D == 3 ? iceil((b.end[2] - b.start[2]) / gs / std::sqrt(6.0) * 3.0) : 1;
    } else {
        ni = iceil((b.end[0] - b.start[0]) / gs);
        nj = iceil((b.end[1] - b.start[1]) / gs);
        nk = D == 3 ? iceil((b.end[2] - b.start[2]) / gs) : 1;
    }
    ni = std::max(ni, 1);
    nj = std::max(nj, 1);
    nk = std::max(nk, 1);
}

void check_square(Geometry &g, Block &b, int &fault) { /* src/shapes/square.cpp:6-96 */
    if (!g.check_vector(b.start)) { g.msg("block \"%s\": start point missing", b.name.c_str()); fault = 1; }
    if (!g.check_vector(b.end)) { g.msg("block \"%s\": end point missing", b.name.c_str()); fault = 1; }
    if (b.dx < 0 && (b.ni < 0 || b.nj < 0)) b.dx = g.gs_running;
    if (b.ni > 0 && b.nj > 0 && (g.D == 2 || b.nk > 0) && b.dx < 0) {
        const V dist = vsub(b.end, b.start);
        const double di = dist[0] / double(b.ni), dj = dist[1] / double(b.nj);
        /* the k spacing divides the y extent upstream */
        b.dx = g.D == 2 ? std::min(di, dj) : std::min(di, std::min(dj, dist[1] / double(b.nk)));
    }
    int ni, nj, nk;
    box_counts(b, g.gs_running, g.D, ni, nj, nk);
    b.ni = ni;
    b.nj = nj;
    if (g.D == 3) b.nk = nk;
    b.npts = (int64_t)ni * nj * (g.D == 3 ? nk : 1);
}

void check_circle(Geometry &g, Block &b, int &fault) { /* src/shapes/circle.cpp:6-95 */
    if (!g.check_vector(b.centre)) { g.msg("block \"%s\": centre missing", b.name.c_str()); fault = 1; }
    if (b.radius < 0) { g.msg("block \"%s\": radius missing", b.name.c_str()); fault = 1; }
    for (int k = 0; k < g.D; ++k) {
        b.start[k] = b.centre[k] - b.radius;
        b.end[k] = b.centre[k] + b.radius;
    }
    if (b.dx < 0) b.dx = b.ni < 0 ? g.gs_running : (2.0 * b.radius) / double(b.ni);
    int ni, nj, nk; /* local counts: the block's own stay untouched */
    box_counts(b, g.gs_running, g.D, ni, nj, nk);
    int npoints = ni * nj * (g.D == 3 ? nk : 1);
    npoints = npoints > 1 ? npoints : 1;
    b.npts = (int64_t)std::ceil(double(npoints) * kPi / (g.D == 2 ? 4.0 : 6.0));
}

/* the normal-only rotation branches of cylinder.cpp:187-217 and inlet.cpp:128-186 build a local
 * matrix that is discarded; their lasting effects are the normalised normal and, in 2D, angles[0] */
void normal_branch(Geometry &g, Block &b, double angle_shift) {
    b.normal = vnormalized(b.normal);
    if (g.D == 2) b.angles[0] = std::atan2(b.normal[1], b.normal[0]) + angle_shift;
}

void check_cylinder(Geometry &g, Block &b, int &fault) { /* src/shapes/cylinder.cpp:7-302 */
    const int D = g.D;
    const double gs = g.gs_running;
    int has_config = 0;
    auto from_centre_radius = [&](void) {
        b.start = b.centre;
        b.start[1] -= b.radius;
        b.end = b.centre;
        b.end[1] += b.radius;
        if (D == 3) {
            b.start[2] -= b.radius;
            b.end[2] += b.radius;
            b.right = b.centre;
            b.right[1] += b.radius;
            b.right[2] -= b.radius;
        }
    };
    auto from_centre_right_end = [&](void) {
        const V v = vsub(b.right, b.centre), u = vsub(b.end, b.right);
        b.start = vsub(vsub(b.centre, v), u);
        b.right = vadd(b.start, vmul(v, 2.0));
        b.end = vadd(b.right, vmul(u, 2.0));
        b.radius = vnorm(v);
    };
    if (b.subshape == "Hollow") {
        b.sub_bound_type = hollow;
        if (b.thickness < 0 && b.nk < 0) { g.msg("cylinder \"%s\": needs a thickness or a wall count", b.name.c_str()); fault = 1; }
        if (b.length < 0 && b.nj < 0) { g.msg("cylinder \"%s\": needs a length or a j count", b.name.c_str()); fault = 1; }
        if (g.check_vector(b.centre)) {
            if (b.radius > 0) {
                has_config = 3;
                from_centre_radius();
            } else if (D == 3 && g.check_vector(b.right) && g.check_vector(b.end)) {
                has_config = 4;
                from_centre_right_end();
            }
        } else if (g.check_vector(b.start) && g.check_vector(b.end) && (D == 2 || g.check_vector(b.right))) {
            has_config = 1;
            b.centre = vmul(vadd(b.start, b.end), 0.5);
            const V v = vsub(b.right, b.start);
            b.radius = 0.5 * vnorm(v);
            b.right = vadd(b.centre, vmul(v, 0.5));
        }
    } else if (b.subshape == "Solid") {
        b.sub_bound_type = solid;
        if (b.length < 0 || b.nk < 0) { g.msg("cylinder \"%s\": needs a length and a k count", b.name.c_str()); fault = 1; }
        if (g.check_vector(b.start) && g.check_vector(b.right) && g.check_vector(b.end)) {
            has_config = 1;
            b.centre = vmul(vadd(b.start, b.end), 0.5);
            b.radius = 0.5 * vnorm(vsub(b.right, b.start));
        } else if (g.check_vector(b.centre)) {
            if (b.radius > 0) {
                has_config = 3;
                from_centre_radius();
            }
            if (g.check_vector(b.right) && g.check_vector(b.end)) {
                has_config = 4;
                from_centre_right_end();
            }
        } else if (g.check_vector(b.start) && b.ni > 0 && b.nj > 0) {
            has_config = 2;
        }
    } else {
        g.msg("cylinder \"%s\": unknown sub type (Hollow or Solid)", b.name.c_str());
        fault = 1;
    }
    if (has_config == 0) { g.msg("cylinder \"%s\": not enough geometry to place it", b.name.c_str()); fault = 1; }

    if (vnorm(b.angles) != 0) {
        b.angles = vmul(b.angles, kPi / 180.0);
        b.rotmat = rotation(b.angles, D);
        b.normal = mv(b.rotmat, V{1, 0, 0});
    } else if (!g.is_unit_x(b.normal)) {
        normal_branch(g, b, 0.0);
    }
    if (has_config == 1) { /* three points define the plane; the matrix built here is discarded */
        const V ab = vnormalized(vsub(b.end, b.start));
        if (D == 3) {
            const V ac = vnormalized(vsub(b.right, b.start));
            b.normal = vnormalized(vcross(ab, ac));
        } else {
            b.angles[0] = std::atan2(ab[1], ab[0]);
            b.normal = V{std::cos(b.angles[0]), -std::sin(b.angles[0]), 0.0};
        }
    }
    if (has_config == 2) {
        b.centre = b.start;
        b.radius = 0.5 * gs * b.ni;
        b.centre[1] += b.radius;
        if (D == 3) {
            b.right = b.start;
            b.right[1] += gs * b.ni;
            b.end = b.right;
            b.end[2] += gs * b.nj;
            b.centre[2] += b.radius;
        } else {
            b.end = b.start;
            b.end[1] += gs * b.ni;
        }
        if (!is_identity(b.rotmat, D)) {
            b.centre = vadd(mv(b.rotmat, vsub(b.centre, b.start)), b.start);
            b.end = vadd(mv(b.rotmat, vsub(b.end, b.start)), b.start);
            if (D == 3) b.right = vadd(mv(b.rotmat, vsub(b.right, b.start)), b.start);
        }
    } else if (has_config == 3 || has_config == 4) {
        if (!is_identity(b.rotmat, D)) {
            b.start = vadd(mv(b.rotmat, vsub(b.start, b.centre)), b.centre);
            b.end = vadd(mv(b.rotmat, vsub(b.end, b.centre)), b.centre);
            if (D == 3) b.right = vadd(mv(b.rotmat, vsub(b.right, b.centre)), b.centre);
        }
    }
    b.dx = gs;
    if (b.sub_bound_type == hollow) {
        if (b.thickness < 0) {
            b.thickness = b.particle_order ? double(b.nk) * gs * std::sqrt(3.0) * 2.0 : double(b.nk) * gs;
        } else if (b.nk < 0) {
            b.nk = b.particle_order ? iceil(b.thickness / (gs * std::sqrt(3.0) * 2.0)) : iceil(b.thickness / gs);
            b.nk = std::max(b.nk, 1);
        }
        if (D == 3) {
            const double dtheta = gs / b.radius;
            b.ni = std::max(iceil((2 * kPi) / dtheta), 1);
        }
        b.nj = std::max(iceil(b.length / gs) + 1, 1);
        b.npts = (int64_t)b.nj * b.nk * (D == 3 ? b.ni : 2);
    } else if (b.sub_bound_type == solid) {
        b.ni = std::max(iceil(2.0 * b.radius / gs), 1);
        b.nj = std::max(iceil(b.length / gs), 1);
        if (D == 3) b.nk = iceil(2.0 * b.radius / gs);
        b.nk = std::max(b.nk, 1);
        if (D == 3) {
            int64_t n = (int64_t)(b.nj * b.nk * (kPi / 4.0) * b.ni);
            b.npts = n * b.ni;
        } else {
            b.npts = (int64_t)b.ni * b.nj;
        }
    }
}

/* 2D arc helpers (src/shapes/arc.cpp:10-79) */
void arc_centrepoint_2d(Geometry &g, Block &b, int &fault) {
    const V d0 = vsub(b.start, b.centre), d1 = vsub(b.end, b.centre);
    const double r = vsq(d0);
    if (std::fabs(vsq(d1) - r) > 0.001) {
        g.msg("arc end point lies at another radius from the centre than the start point");
        fault = 1;
        return;
    }
    b.radius = std::sqrt(r);
    b.arc_start = std::atan2(d0[1], d0[0]) * 180 / kPi;
    b.arc_end = std::atan2(d1[1], d1[0]) * 180 / kPi;
}

/* solve a 2x2 system m x = v (Gaussian elimination with partial pivoting) */
bool solve2(double m00, double m01, double m10, double m11, double v0, double v1, double &x0, double &x1) {
    if (std::fabs(m10) > std::fabs(m00)) {
        std::swap(m00, m10);
        std::swap(m01, m11);
        std::swap(v0, v1);
    }
    if (m00 == 0.0) return false;
    const double f = m10 / m00;
    const double a11 = m11 - f * m01, w1 = v1 - f * v0;
    if (a11 == 0.0) return false;
    x1 = w1 / a11;
    x0 = (v0 - m01 * x1) / m00;
    return true;
}

void arc_midpoint_2d(Geometry &g, Block &b, int &fault) {
    const V &s = b.start, &e = b.end, &mp = b.mid;
    const double r1x = s[0] * s[0], r1y = s[1] * s[1], r2x = mp[0] * mp[0], r2y = mp[1] * mp[1];
    const double r3x = e[0] * e[0], r3y = e[1] * e[1];
    double cx = 0, cy = 0;
    if (!solve2(2.0 * (s[0] - e[0]), 2.0 * (s[1] - e[1]), 2.0 * (s[0] - mp[0]), 2.0 * (s[1] - mp[1]),
                r1x - r3x + r1y - r3y, r1x - r2x + r1y - r2y, cx, cy)) {
        g.msg("block \"%s\": the three arc points lie on one line", b.name.c_str());
        fault = 1;
        return;
    }
    b.centre = V{cx, cy, 0.0};
    arc_centrepoint_2d(g, b, fault);
}

/* 3D arch helpers (src/shapes/arc.cpp:164-277) */
void arc_end_3d(Geometry &g, Block &b, int &fault) {
    V u = vsub(b.start, b.centre);
    b.radius = vnorm(u);
    u = vdiv(u, b.radius);
    const V w = vnormalized(b.right);
    if (std::fabs(vdot(b.right, b.start) - vdot(b.right, b.centre)) > 1e-4) {
        g.msg("arc points are not in the plane of the given normal");
        fault = 1;
        return;
    }
    const V v = vnormalized(vcross(u, w));
    const double alen = b.arclength * kPi / 180.0;
    b.end = vadd(vmul(vadd(vmul(u, std::cos(alen)), vmul(v, std::sin(alen))), b.radius), b.centre);
}

void arc_centrepoint_3d(Geometry &g, Block &b, int &fault) {
    V d1 = vsub(b.start, b.centre), d2 = vsub(b.end, b.centre);
    const double r = vsq(d1);
    if (std::fabs(vsq(d2) - r) > 0.001) {
        g.msg("arc end point lies at another radius from the centre than the start point");
        fault = 1;
        return;
    }
    b.radius = std::sqrt(r);
    d1 = vnormalized(d1);
    d2 = vnormalized(d2);
    const V w = vnormalized(vcross(d2, d1));
    const V v = vnormalized(vcross(w, d1));
    const double maxx = std::fabs(d1[0]) + std::fabs(v[0]);
    const double maxy = std::fabs(d1[1]) + std::fabs(v[1]);
    const double maxz = std::fabs(d1[2]) + std::fabs(v[2]);
    int r0 = 0, r1 = 1;
    if (maxx < maxy && maxx < maxz) { r0 = 1; r1 = 2; }
    else if (maxy < maxx && maxy < maxz) { r0 = 0; r1 = 2; }
    /* the right-hand side stays (v_x, v_y) in every case: upstream's attempt to reassign it
     * (`v_(v[1], v[2])`) reads two coefficients and discards them */
    double a = 0, bb = 0;
    solve2(d1[r0], v[r0], d1[r1], v[r1], v[0], v[1], a, bb);
    b.arc_start = std::atan2(1.0, 0.0) * 180 / kPi;
    b.arc_end = std::atan2(a, bb) * 180 / kPi;
    b.right = w;
}

void check_arc(Geometry &g, Block &b, int &fault) { /* src/shapes/arc.cpp:364-553 */
    const int D = g.D;
    const double gs = g.gs_running;
    int has_config = 0, arc_defined = 0;
    if (D == 2 && g.check_vector(b.centre)) {
        if (b.arc_start >= 0 && b.arc_end >= 0 && b.radius > 0) has_config = 1;
        else if (b.arc_start >= 0 && b.ni > 0 && b.radius > 0) has_config = 1;
        else if (b.arc_start >= 0 && b.arclength != kDefault && b.radius > 0) { has_config = 1; arc_defined = 1; }
    }
    if (!has_config && g.check_vector(b.centre) && g.check_vector(b.start) && g.check_vector(b.end)) {
        has_config = 1;
        if (D == 2) arc_centrepoint_2d(g, b, fault);
        else arc_centrepoint_3d(g, b, fault);
    }
    if (!has_config) {
        if (D == 3) {
            if (g.check_vector(b.centre) && g.check_vector(b.start) && g.check_vector(b.mid) && b.arclength != kDefault) {
                has_config = 1;
                arc_defined = 1;
            }
        } else if (g.check_vector(b.start) && g.check_vector(b.end) && g.check_vector(b.mid)) {
            has_config = 1;
            arc_midpoint_2d(g, b, fault);
        }
    }
    if (!has_config && g.check_vector(b.centre) && g.check_vector(b.start) && b.arclength != kDefault) {
        if (D == 2 || g.check_vector(b.right)) {
            has_config = 1;
            arc_defined = 1;
        }
    }
    if (!has_config) { g.msg("block \"%s\": not enough arc geometry to place it", b.name.c_str()); fault = 1; }
    if (b.dx < 0) b.dx = b.ni < 0 ? gs : (2.0 * b.radius) / double(b.ni);
    if (b.thickness < 0) {
        if (b.nk < 0) { g.msg("block \"%s\": arc wall thickness or layer count missing", b.name.c_str()); fault = 1; }
    } else if (b.nk < 0) {
        b.nk = b.particle_order ? iceil(b.thickness / gs / std::sqrt(3.0) * 2.0) : iceil(b.thickness / gs);
    }
    const double dtheta = gs / b.radius;
    if (arc_defined) {
        if (D == 3) arc_end_3d(g, b, fault);
    } else {
        if (b.arc_end < 0 && b.ni > 0) b.arc_end = 180.0 / kPi * (b.arc_start * kPi / 180 + double(b.ni) * dtheta);
        b.arclength = b.arc_end - b.arc_start;
    }
    /* a local count: the block's own ni (used by the 2D generator) is left as read */
    const int ni = std::max(iceil((std::fabs(b.arclength) * kPi / 180) / dtheta), 1);
    const int smax = b.sstraight > 0 ? iceil(b.sstraight / gs) : 0;
    const int emax = b.estraight > 0 ? iceil(b.estraight / gs) : 0;
    b.npts = (int64_t)(ni + smax + emax) * b.nk;
    if (D == 3) {
        if (b.length < 0) {
            if (b.nj < 0) { g.msg("block \"%s\": arch length or j count missing", b.name.c_str()); fault = 1; }
        } else if (b.nj < 0) {
            b.nj = b.particle_order ? iceil(b.length / gs / std::sqrt(6.0) * 3.0) : iceil(b.length / gs);
            b.nj = std::max(b.nj, 1);
        }
        b.npts *= b.nj;
    }
}

void check_inlet(Geometry &g, Block &b, int &fault) { /* src/shapes/inlet.cpp:7-263 */
    const int D = g.D;
    const double gs = g.gs_running;
    int has_config = 0;
    if (D == 3) {
        if (b.subshape == "Square") {
            b.sub_bound_type = squareCube;
            if (g.check_vector(b.start) && g.check_vector(b.right) && g.check_vector(b.end)) has_config = 1;
            if (g.check_vector(b.start) && b.ni > 0 && b.nj > 0) has_config = 2;
        } else if (b.subshape == "Circle") {
            b.sub_bound_type = circleSphere;
            if (g.check_vector(b.centre)) {
                if (g.check_vector(b.right) && g.check_vector(b.end)) {
                    has_config = 4;
                    const V v = vsub(b.right, b.centre), u = vsub(b.end, b.right);
                    b.start = vsub(vsub(b.centre, v), u);
                    b.right = vadd(b.start, vmul(v, 2.0));
                    b.end = vadd(b.right, vmul(u, 2.0));
                }
                if (b.radius > 0) {
                    has_config = 3;
                    b.start = b.centre;
                    b.start[1] -= b.radius;
                    b.start[2] -= b.radius;
                    b.end = b.centre;
                    b.end[1] += b.radius;
                    b.end[2] += b.radius;
                    b.right = b.centre;
                    b.right[1] += b.radius;
                    b.right[2] -= b.radius;
                }
            } else if (g.check_vector(b.start) && g.check_vector(b.right) && g.check_vector(b.end)) {
                has_config = 1;
                b.centre = vmul(vadd(b.start, b.end), 0.5);
                const V v = vsub(b.right, b.start);
                b.radius = 0.5 * vnorm(v);
                b.right = vadd(b.centre, vmul(v, 0.5));
            }
        } else {
            g.msg("inlet \"%s\": unknown section shape", b.name.c_str());
            fault = 1;
        }
    } else {
        if (g.check_vector(b.start) && g.check_vector(b.end)) {
            has_config = 1;
            b.centre = vmul(vadd(b.start, b.end), 0.5);
            b.radius = vnorm(vsub(b.centre, b.start));
        } else if (g.check_vector(b.centre) && b.radius > 0) {
            has_config = 3;
            b.start = b.centre;
            b.start[1] -= b.radius;
            b.end = b.centre;
            b.end[1] += b.radius;
        }
    }
    if (has_config == 0) { g.msg("inlet \"%s\": not enough geometry to place it", b.name.c_str()); fault = 1; }
    b.dx = gs;
    if (vnorm(b.angles) != 0) {
        b.angles = vmul(b.angles, kPi / 180.0);
        b.rotmat = rotation(b.angles, D);
        b.normal = mv(b.rotmat, V{1, 0, 0});
        b.insert_norm = b.normal;
    } else if (!g.is_unit_x(b.normal)) {
        normal_branch(g, b, 0.0);
        b.insert_norm = b.normal;
    } else if (!g.is_unit_x(b.insert_norm)) {
        b.normal = b.insert_norm;
        normal_branch(g, b, -kPi / 2.0);
    }
    if (has_config == 1) { /* the matrix built here is discarded */
        const V ab = vnormalized(vsub(b.end, b.start));
        if (D == 3) {
            const V ac = vnormalized(vsub(b.right, b.start));
            b.normal = vnormalized(vcross(ab, ac));
        } else {
            b.angles[0] = std::atan2(ab[1], ab[0]);
            b.normal = V{std::sin(b.angles[0]), std::cos(b.angles[0]), 0.0};
        }
        b.insert_norm = b.normal;
        const V test = vsub(b.start, vmul(b.insert_norm, b.length - 0.01 * gs));
        b.insconst = vdot(b.insert_norm, test);
    } else if (has_config == 2) {
        if (D == 3) {
            b.right = b.start;
            b.right[1] += gs * b.ni;
            b.end = b.right;
            b.end[2] += gs * b.nj;
        } else {
            b.end = b.start;
            b.end[1] += gs * b.ni;
        }
        if (!is_identity(b.rotmat, D)) {
            b.end = vadd(mv(b.rotmat, vsub(b.end, b.start)), b.start);
            if (D == 3) b.right = vadd(mv(b.rotmat, vsub(b.right, b.start)), b.start);
        }
    } else if (has_config == 3 || has_config == 4) {
        if (!is_identity(b.rotmat, D)) {
            b.start = vadd(mv(b.rotmat, vsub(b.start, b.centre)), b.centre);
            b.end = vadd(mv(b.rotmat, vsub(b.end, b.centre)), b.centre);
            if (D == 3) b.right = vadd(mv(b.rotmat, vsub(b.right, b.centre)), b.centre);
        }
    }
    const double xlength = D == 3 ? vnorm(vsub(b.right, b.start)) : vnorm(vsub(b.end, b.start));
    b.ni = std::max(iceil(xlength / gs), 1);
    if (D == 3) b.nj = std::max(iceil(vnorm(vsub(b.end, b.right)) / gs), 1);
    b.nk = std::max(iceil(b.length / gs), 1);
    const int nBuff = 4;
    if (D == 3) {
        if (b.sub_bound_type == circleSphere) {
            if (!g.check_vector(b.centre)) b.centre = vmul(vadd(b.start, b.end), 0.5);
            if (b.radius < 0) b.radius = vnorm(vsub(b.centre, b.start)) * std::cos(kPi / 4.0);
            b.npts = (int64_t)(b.ni * b.nj * (kPi / 4.0) * (b.nk + nBuff + 1));
        } else {
            b.npts = (int64_t)b.ni * b.nj * (b.nk + nBuff + 1);
        }
    } else {
        b.npts = (int64_t)b.ni * (b.nk + nBuff);
    }
    if (b.vmag != 0) b.vel = vmul(b.insert_norm, b.vmag);
}

void check_coords(Geometry &g, Block &b, int &fault) { /* src/shapes/coordinates.cpp:8-29 */
    if (b.filename.empty()) {
        if (b.coords.empty()) {
            g.msg("block \"%s\": coordinate list is incomplete", b.name.c_str());
            fault = 1;
        } else {
            b.npts = (int64_t)b.coords.size();
        }
    }
}

void check_input(Geometry &g, Block &b, int &fault) {
    check_base(g, b, fault);
    switch (b.bound_type) {
    case linePlane: check_line(g, b, fault); break;
    case squareCube: check_square(g, b, fault); break;
    case circleSphere: check_circle(g, b, fault); break;
    case cylinder: check_cylinder(g, b, fault); break;
    case arcSection: check_arc(g, b, fault); break;
    case inletZone: check_inlet(g, b, fault); break;
    case coordDef: check_coords(g, b, fault); break;
    default: return; /* unrecognised shape: reported already, no post step (no override upstream) */
    }
    check_post(g, b);
}

/* ---- generate_points ------------------------------------------------------------------------ */

struct Draw { /* uniform_real_distribution(0, eps * dx) over a default-constructed engine */
    std::default_random_engine re;
    std::uniform_real_distribution<double> unif;
    explicit Draw(double dx) : unif(0.0, kEps * dx) {}
    double operator()() { return unif(re); }
    V one(int D) { /* StateVecD::Constant(unif(re)): one draw on every component */
        const double u = unif(re);
        return V{u, u, D == 3 ? u : 0.0};
    }
    V each(int D) { /* StateVecD(unif(re), unif(re)[, unif(re)]) */
        V r{0, 0, 0};
        for (int k = 0; k < D; ++k) r[k] = unif(re);
        return r;
    }
};

void gen_line(const Geometry &g, Block &b, double gs) { /* src/shapes/line.cpp:127-188 */
    Draw U(gs);
    const double s3 = std::sqrt(3.0), s6 = std::sqrt(6.0);
    if (g.D == 2) {
        const V delta = vmul(vnormalized(vsub(b.end, b.start)), gs);
        const V norm{delta[1], -delta[0], 0.0};
        for (int ii = 0; ii < b.ni; ++ii)
            for (int jj = 0; jj < b.nk; ++jj) {
                V p;
                if (b.particle_order)
                    p = vadd(vmul(delta, double(ii + 0.5 * (jj % 2))), vmul(vmul(vmul(norm, 0.5), s3), double(jj)));
                else
                    p = vadd(vmul(delta, double(ii)), vmul(norm, double(jj)));
                p = vadd(p, U.one(2));
                p = vadd(p, b.start);
                b.coords.push_back(p);
            }
        return;
    }
    const V di = vmul(vnormalized(vsub(b.right, b.start)), gs);
    const V dj = vmul(vnormalized(vsub(b.end, b.right)), gs);
    const V norm = vmul(vnormalized(vcross(dj, di)), gs);
    for (int jj = 0; jj < b.nj; ++jj)
        for (int ii = 0; ii < b.ni; ++ii)
            for (int kk = 0; kk < b.nk; ++kk) {
                V p;
                if (b.particle_order)
                    p = vmul(vadd(vadd(vmul(di, double(2 * ii + ((jj + kk) % 2))),
                                       vmul(dj, s3 * (double(jj) + double(kk % 2) / 3))),
                                  vmul(vdiv(vmul(vmul(norm, 2.0), s6), 3.0), double(kk))),
                             0.5);
                else
                    p = vadd(vadd(vmul(di, double(ii)), vmul(dj, double(jj))), vmul(norm, double(kk)));
                p = vadd(p, U.one(3));
                p = vadd(p, b.start);
                b.coords.push_back(p);
            }
}

/* lattice point of a box (square.cpp:116-128, circle.cpp:153-162), before scaling by dx */
V lattice(bool hcp, int D, int i, int j, int k) {
    if (D == 2)
        return hcp ? vmul(V{double(2 * i + (j % 2)), std::sqrt(3.0) * double(j), 0.0}, 0.5)
                   : V{double(i), double(j), 0.0};
    return hcp ? vmul(V{double(2 * i + ((j + k) % 2)), std::sqrt(3.0) * (double(j) + double(k % 2) / 3.0),
                        2.0 / 3.0 * std::sqrt(6.0) * double(k)},
                      0.5)
               : V{double(i), double(j), double(k)};
}

void gen_square(const Geometry &g, Block &b, double gs) { /* src/shapes/square.cpp:98-146 */
    Draw U(gs);
    const int nk = g.D == 3 ? b.nk : 1;
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < b.nj; ++j)
            for (int i = 0; i < b.ni; ++i) {
                V p = vmul(lattice(b.particle_order, g.D, i, j, k), gs);
                p = vadd(p, U.one(g.D));
                p = vadd(p, b.start);
                b.coords.push_back(p);
            }
}

/* rings of points from the radius inwards, then the centre (circle.cpp:98-135,
 * inlet.cpp:383-421); `at` places a ring point (a, c) in the block's frame */
template <typename F>
void rings(double radius, double gs, F &&at) {
    for (double rad = radius; rad > 0.99 * gs; rad -= gs) {
        double dtheta = std::atan(gs / rad);
        const int ncirc = (int)std::floor(std::fabs(2.0 * kPi / dtheta));
        dtheta = 2.0 * kPi / double(ncirc);
        for (double theta = 0.0; theta < 2 * kPi - 0.5 * dtheta; theta += dtheta)
            at(rad * std::sin(theta), rad * std::cos(theta));
    }
}

void gen_circle(const Geometry &g, Block &b, double gs) { /* src/shapes/circle.cpp:97-196 */
    Draw U(gs);
    if (g.D == 2) {
        rings(b.radius, gs, [&](double x, double y) {
            V p = vadd(V{x, y, 0.0}, U.each(2));
            p = mv(b.rotmat, p);
            b.coords.push_back(vadd(p, b.centre));
        });
        V p = U.each(2);
        p = mv(b.rotmat, p);
        b.coords.push_back(vadd(p, b.centre));
        return;
    }
    const double rsq = b.radius * b.radius;
    int ni, nj, nk;
    box_counts(b, gs, 3, ni, nj, nk);
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) {
                V p = vmul(lattice(b.particle_order, 3, i, j, k), gs);
                p = mv(b.rotmat, p);
                p = vadd(p, U.each(3));
                p = vadd(p, b.start);
                if (vsq(vsub(p, b.centre)) > rsq) continue;
                b.coords.push_back(p);
            }
}

void gen_cylinder(const Geometry &g, Block &b, double gs) { /* src/shapes/cylinder.cpp:304-528 */
    /* solid cylinders generate nothing upstream: their loops run while ii > ni (2D) or
     * kk > nk (3D) from zero */
    if (b.sub_bound_type != hollow) return;
    Draw U(gs);
    if (g.D == 2) {
        const V norm = vnormalized(b.normal);
        const V left{norm[1], -norm[0], 0.0};
        const double r = b.radius, s3 = std::sqrt(3.0);
        for (int side = 0; side < 2; ++side) {
            const double sg = side == 0 ? 1.0 : -1.0;
            for (int ii = 0; ii < b.nj; ++ii)
                for (int kk = 0; kk < b.nk; ++kk) {
                    V p;
                    if (b.particle_order)
                        p = vmul(vadd(vmul(norm, double(-ii + 0.5 * (kk % 2))), vmul(vmul(vmul(left, 0.5), s3), sg * double(kk))), gs);
                    else
                        p = vmul(vadd(vmul(norm, double(-ii)), vmul(left, sg * double(kk))), gs);
                    p = vadd(p, vmul(left, sg * r));
                    p = vadd(p, U.each(2));
                    p = vadd(p, b.centre);
                    b.coords.push_back(p);
                }
        }
        return;
    }
    const double dtheta = 2 * kPi / double(b.ni);
    for (int jj = 0; jj < b.nj; jj++)
        for (int kk = 0; kk < b.nk; kk++) {
            double r = b.radius, l = double(jj) * gs, doffset = 0;
            if (b.particle_order) {
                r += 1.0 / 3.0 * std::sqrt(6.0) * double(kk) * gs;
                l = 0.5 * std::sqrt(3.0) * (double(jj) + double(kk % 2) / 3.0) * gs;
                doffset = 0.5 * dtheta * ((kk + jj) % 2);
            } else {
                r += double(kk) * gs;
            }
            for (int ii = 0; ii < b.ni; ii++) {
                double theta = double(ii) * dtheta;
                if (b.particle_order) theta += doffset;
                V p{-l, std::cos(theta) * r, std::sin(theta) * r};
                p = vadd(p, U.each(3));
                p = mv(b.rotmat, p);
                b.coords.push_back(vadd(p, b.centre));
            }
        }
}

void gen_arc(const Geometry &g, Block &b, double gs) { /* src/shapes/arc.cpp:81-160, 279-357, 555-580 */
    Draw U(gs);
    if (g.D == 2) {
        const double theta0 = b.arc_start * kPi / 180.0, dtheta = gs / b.radius;
        const int ni = b.ni, nk = b.nk; /* the block's ni as read (see check_arc) */
        const V svec{std::cos(theta0), std::sin(theta0), 0.0};
        const V snormal{svec[1], -svec[0], 0.0};
        const int smax = iceil(b.sstraight / gs);
        const V evec{std::cos(theta0 + double(ni - 1) * dtheta), std::sin(theta0 + double(ni - 1) * dtheta), 0.0};
        const V enormal{-evec[1], evec[0], 0.0};
        const int emax = iceil(b.estraight / gs);
        for (int jj = 0; jj < nk; jj++) {
            if (b.sstraight > 0)
                for (int ii = smax; ii > 0; ii--) {
                    V p = vadd(vmul(svec, b.radius - double(jj) * gs), vmul(snormal, double(ii) * gs));
                    p = vadd(p, vadd(U.each(2), b.centre));
                    b.coords.push_back(p);
                }
            for (int ii = 0; ii < ni; ii++) {
                double theta = theta0 + double(ii) * dtheta, r = b.radius;
                if (b.particle_order) {
                    theta += 0.5 * dtheta * (jj % 2);
                    r -= 0.5 * std::sqrt(3.0) * double(jj) * gs;
                } else {
                    r -= double(jj) * gs;
                }
                V p{std::cos(theta) * r, std::sin(theta) * r, 0.0};
                p = vadd(p, U.each(2));
                b.coords.push_back(vadd(p, b.centre));
            }
            if (b.estraight > 0)
                for (int ii = 1; ii <= emax; ii++) {
                    V p = vadd(vmul(evec, b.radius - double(jj) * gs), vmul(enormal, double(ii) * gs));
                    p = vadd(p, vadd(U.each(2), b.centre));
                    b.coords.push_back(p);
                }
        }
        return;
    }
    const double dtheta = gs / b.radius;
    const int nrad = iceil(b.arclength * kPi / 180.0 / dtheta);
    const V u = vnormalized(vsub(b.start, b.centre));
    const V w = vnormalized(b.right);
    const V v = vnormalized(vcross(u, w));
    const int smax = iceil(b.sstraight / gs), emax = iceil(b.estraight / gs);
    const V evec = vadd(vmul(u, std::cos(double(nrad - 1) * dtheta)), vmul(v, std::sin(double(nrad - 1) * dtheta)));
    const V enorm = vcross(evec, w);
    for (int kk = 0; kk < b.nj; kk++)
        for (int jj = 0; jj < b.nk; jj++) {
            double r = b.radius, l = double(kk) * gs, doffset = 0;
            if (b.particle_order) {
                r += 1.0 / 3.0 * std::sqrt(6.0) * double(jj) * gs;
                l = 0.5 * std::sqrt(3.0) * (double(kk) + double(jj % 2) / 3.0) * gs;
                doffset = 0.5 * dtheta * ((jj + kk) % 2);
            } else {
                r += double(jj) * gs;
            }
            if (b.sstraight > 0)
                for (int ii = smax; ii > 0; ii--) {
                    const double dist = double(ii) * gs + doffset;
                    V p = vadd(vsub(vmul(u, r), vmul(v, dist)), vmul(w, l));
                    p = vadd(p, vadd(U.each(3), b.centre));
                    b.coords.push_back(p);
                }
            for (int ii = 0; ii < nrad; ii++) {
                double theta = double(ii) * dtheta;
                const double la = double(kk) * gs; /* the arc itself uses the unshifted layer offset */
                if (b.particle_order) theta += doffset;
                V p = vadd(vadd(vmul(u, std::cos(theta) * r), vmul(v, std::sin(theta) * r)), vmul(w, la));
                p = vadd(p, U.each(3));
                b.coords.push_back(vadd(p, b.centre));
            }
            if (b.estraight > 0)
                for (int ii = 1; ii <= emax; ii++) {
                    const double dist = double(ii) * gs + doffset;
                    V p = vadd(vadd(vmul(evec, r), vmul(enorm, dist)), vmul(w, l));
                    p = vadd(p, vadd(U.each(3), b.centre));
                    b.coords.push_back(p);
                }
        }
}

/* one inlet disk of the 3D circular inlet at depth kk (inlet.cpp:380-460); a fresh engine each */
std::vector<V> inlet_disk(const Block &b, double dx, int kk) {
    Draw U(dx);
    std::vector<V> pts;
    if (b.particle_order) {
        const double x = -dx * kk;
        rings(b.radius, dx, [&](double y, double z) {
            V p = vadd(V{x, y, z}, U.each(3));
            p = mv(b.rotmat, p);
            pts.push_back(vadd(p, b.centre));
        });
        V p = vadd(V{x, 0.0, 0.0}, U.each(3));
        p = mv(b.rotmat, p);
        pts.push_back(vadd(p, b.centre));
        return pts;
    }
    const double rsq = b.radius * b.radius;
    for (int jj = 0; jj < b.nj; ++jj)
        for (int ii = 0; ii < b.ni; ++ii) {
            V p = vmul(V{-double(kk), double(ii), double(jj)}, dx);
            const double a = p[1] - b.radius, c = p[2] - b.radius;
            if (a * a + c * c > rsq) continue;
            p = vadd(p, U.each(3));
            p = mv(b.rotmat, p);
            pts.push_back(vadd(p, b.start));
        }
    return pts;
}

void gen_inlet(const Geometry &g, Block &b, double gs) { /* src/shapes/inlet.cpp:265-575 */
    const int nBuff = 4;
    auto add = [&](const V &p, int type) {
        b.coords.push_back(p);
        b.bc.push_back(type);
    };
    if (g.D == 2) {
        Draw U(gs);
        const V delta = vdiv(vsub(b.end, b.start), double(b.ni));
        const V norm{delta[1], -delta[0], 0.0};
        auto at = [&](int ii, int jj) {
            V p = vadd(vmul(delta, double(ii)), vmul(norm, double(-jj)));
            p = vadd(p, U.one(2));
            return vadd(p, b.start);
        };
        for (int jj = 0; jj < b.nk; ++jj)
            for (int ii = 0; ii < b.ni; ++ii) add(at(ii, jj), FJSPH_PIPE);
        for (int ii = 0; ii < b.ni; ++ii) {
            add(at(ii, b.nk), FJSPH_BACK);
            b.back.push_back((int64_t)b.coords.size() - 1);
        }
        b.buffer.assign((size_t)b.ni, std::vector<int64_t>(nBuff, 0));
        for (int jj = b.nk + 1, buff = 0; jj <= b.nk + nBuff; ++jj, ++buff)
            for (int ii = 0; ii < b.ni; ++ii) {
                add(at(ii, jj), FJSPH_BUFFER);
                b.buffer[(size_t)ii][(size_t)buff] = (int64_t)b.coords.size() - 1;
            }
        return;
    }
    if (b.sub_bound_type == squareCube) {
        Draw U(gs);
        auto at = [&](double x, double y, double z) {
            V p = vmul(V{x, y, z}, gs);
            p = vadd(p, U.each(3));
            p = mv(b.rotmat, p);
            return vadd(p, b.start);
        };
        for (int kk = 0; kk < b.nk; ++kk)
            for (int jj = 0; jj < b.nj; ++jj)
                for (int ii = 0; ii < b.ni; ++ii) add(at(-kk, ii, jj), FJSPH_PIPE);
        /* the back layer swaps the in-plane indices: (-nk, jj, ii) */
        for (int jj = 0; jj < b.nj; ++jj)
            for (int ii = 0; ii < b.ni; ++ii) {
                add(at(-b.nk, jj, ii), FJSPH_BACK);
                b.back.push_back((int64_t)b.coords.size() - 1);
            }
        b.buffer.assign(b.back.size(), std::vector<int64_t>(nBuff, 0));
        for (int kk = b.nk + 1, buff = 0; kk <= b.nk + nBuff; ++kk, ++buff) {
            size_t id = 0;
            for (int jj = 0; jj < b.nj; ++jj)
                for (int ii = 0; ii < b.ni; ++ii) {
                    add(at(-kk, ii, jj), FJSPH_BUFFER);
                    b.buffer[id++][(size_t)buff] = (int64_t)b.coords.size() - 1;
                }
        }
    } else if (b.sub_bound_type == circleSphere) {
        for (int kk = 0; kk < b.nk; ++kk)
            for (const V &p : inlet_disk(b, gs, kk)) add(p, FJSPH_PIPE);
        for (const V &p : inlet_disk(b, gs, b.nk)) {
            b.back.push_back((int64_t)b.coords.size());
            add(p, FJSPH_BACK);
        }
        b.buffer.assign(b.back.size(), std::vector<int64_t>(nBuff, 0));
        for (int kk = b.nk + 1, buff = 0; kk <= b.nk + nBuff; ++kk, ++buff) {
            const std::vector<V> disk = inlet_disk(b, gs, kk);
            for (size_t ii = 0; ii < disk.size(); ii++) {
                b.buffer[ii][(size_t)buff] = (int64_t)b.coords.size();
                add(disk[ii], FJSPH_BUFFER);
            }
        }
    }
}

void generate(const Geometry &g, Block &b) {
    const double gs = g.s.dx; /* Generate_Points passes svar.dx */
    switch (b.bound_type) {
    case linePlane: gen_line(g, b, gs); break;
    case squareCube: gen_square(g, b, gs); break;
    case circleSphere: gen_circle(g, b, gs); break;
    case cylinder: gen_cylinder(g, b, gs); break;
    case arcSection: gen_arc(g, b, gs); break;
    case inletZone: gen_inlet(g, b, gs); break;
    default: break; /* coordinates: given with the block (a coordinate file is never read upstream) */
    }
}

/* ---- Check_Intersection (src/Init.cpp:61-233) ------------------------------------------------ */

/* fixed-radius search over one block's points: a uniform grid of cells with edge r, 3^D cells per
 * query; a point matches when its squared distance (accumulated x, y[, z]) is below r^2 */
struct Grid {
    const std::vector<V> *pts = nullptr;
    int D = 2;
    double h = 1, r2 = 1;
    V lo{0, 0, 0};
    std::unordered_map<uint64_t, std::vector<uint32_t>> cells;

    static uint64_t key(int64_t a, int64_t b, int64_t c) {
        return ((uint64_t)(a & 0x1FFFFF) << 42) | ((uint64_t)(b & 0x1FFFFF) << 21) | (uint64_t)(c & 0x1FFFFF);
    }
    int64_t cell(double x, int k) const { return (int64_t)std::floor((x - lo[k]) / h); }
    void build(const std::vector<V> &p, int dim, double r2_) {
        pts = &p;
        D = dim;
        r2 = r2_;
        h = std::sqrt(r2_);
        if (!(h > 0)) h = 1;
        lo = V{0, 0, 0};
        if (!p.empty()) {
            lo = p[0];
            for (const V &x : p)
                for (int k = 0; k < D; ++k) lo[k] = std::min(lo[k], x[k]);
        }
        cells.clear();
        for (size_t i = 0; i < p.size(); ++i)
            cells[key(cell(p[i][0], 0), cell(p[i][1], 1), D == 3 ? cell(p[i][2], 2) : 0)].push_back((uint32_t)i);
    }
    template <typename F>
    void query(const V &q, F &&hit) const {
        const int64_t c0 = cell(q[0], 0), c1 = cell(q[1], 1), c2 = D == 3 ? cell(q[2], 2) : 0;
        const int zr = D == 3 ? 1 : 0;
        for (int64_t a = c0 - 1; a <= c0 + 1; ++a)
            for (int64_t b = c1 - 1; b <= c1 + 1; ++b)
                for (int64_t c = c2 - zr; c <= c2 + zr; ++c) {
                    auto it = cells.find(key(a, b, c));
                    if (it == cells.end()) continue;
                    for (uint32_t j : it->second) {
                        const V &x = (*pts)[j];
                        double d2 = 0;
                        for (int k = 0; k < D; ++k) {
                            const double d = q[k] - x[k];
                            d2 += d * d;
                        }
                        if (d2 < r2) hit(j);
                    }
                }
    }
};

void check_intersection(Geometry &g) {
    const double search = (0.9 * g.s.dx) * (0.9 * g.s.dx);
    auto &bv = g.bound;
    auto &fv = g.fluid;
    for (Block &b : bv) b.intersect.assign(b.coords.size(), 0);
    Grid tree;
    for (size_t id = 0; id < bv.size(); ++id) {
        tree.build(bv[id].coords, g.D, search);
        /* upper triangle including the block itself; a match whose index equals the query's own
         * index is skipped in every block pair, not only within the block */
        for (size_t ii = id; ii < bv.size(); ++ii)
            for (size_t jj = 0; jj < bv[ii].coords.size(); ++jj)
                if (bv[ii].intersect[jj] == 0)
                    tree.query(bv[ii].coords[jj], [&](uint32_t m) {
                        if (m != jj) bv[id].intersect[m] = 1;
                    });
    }
    for (Block &b : fv) b.intersect.assign(b.coords.size(), 0);
    for (size_t id = 0; id < fv.size(); ++id) {
        tree.build(fv[id].coords, g.D, search);
        for (size_t ii = 0; ii < bv.size(); ++ii)
            for (size_t jj = 0; jj < bv[ii].coords.size(); ++jj)
                if (bv[ii].intersect[jj] == 0) tree.query(bv[ii].coords[jj], [&](uint32_t m) { fv[id].intersect[m] = 1; });
        for (size_t ii = id + 1; ii < fv.size(); ++ii)
            for (size_t jj = 0; jj < fv[ii].coords.size(); ++jj)
                if (fv[ii].intersect[jj] == 0) tree.query(fv[ii].coords[jj], [&](uint32_t m) { fv[id].intersect[m] = 1; });
    }
    for (Block &b : fv)
        for (size_t k = 0; k < b.back.size(); ++k) {
            bool hit = b.intersect[(size_t)b.back[k]] != 0;
            for (int64_t q : b.buffer[k]) hit = hit || b.intersect[(size_t)q] != 0;
            if (hit) {
                b.intersect[(size_t)b.back[k]] = 1;
                for (int64_t q : b.buffer[k]) b.intersect[(size_t)q] = 1;
            }
        }
    for (auto *set : {&bv, &fv})
        for (Block &b : *set) b.kept = std::count(b.intersect.begin(), b.intersect.end(), 0);
}

/* ---- Init_Particles (src/Init.cpp:268-494) --------------------------------------------------- */

double eos_density(const fjsph_settings &s, double p) {
    if (s.pressure_rel == FJSPH_ISO_EOS) return (p - s.press_back) / (s.speed_sound * s.speed_sound) + s.rho_rest;
    return s.rho_rest * std::pow(((p - s.press_back) / s.B) + 1.0, 1.0 / s.gam);
}

int assemble(Geometry &g) {
    const fjsph_settings &s = g.s;
    g.xi.clear(); g.v.clear(); g.rho.clear(); g.p.clear(); g.m.clear(); g.b.clear();
    g.limits.clear();
    g.inlets.clear();
    int64_t id = 0;
    auto push = [&](const V &x, const Block &blk, double mass, int type) {
        g.xi.push_back(x);
        g.v.push_back(blk.vel);
        g.rho.push_back(blk.dens);
        g.p.push_back(blk.press);
        g.m.push_back(mass);
        g.b.push_back(type);
        ++id;
    };
    auto base_limits = [&](const Block &blk, bool fluid) {
        fjsph_block L{};
        L.first = id;
        L.is_fluid = fluid ? 1 : 0;
        L.bound_solver = blk.bound_solver;
        L.no_slip = blk.no_slip ? 1 : 0;
        L.block_type = blk.bound_type;
        L.fixed_vel_or_dynamic = blk.fixed_vel_or_dynamic;
        for (int k = 0; k < 3; ++k) {
            L.delete_norm[k] = L.insert_norm[k] = L.aero_norm[k] = kDefault;
        }
        L.delconst = L.insconst = L.aeroconst = kDefault;
        return L;
    };
    auto set_times = [&](fjsph_block &L, const Block &blk, const std::vector<V> &vels, const V &v0) {
        if (!blk.times.empty()) {
            if ((size_t)blk.ntimes > FJSPH_MAX_TIMES || vels.size() > FJSPH_MAX_TIMES) {
                g.msg("block \"%s\": %lld motion times, more than the %d supported", blk.name.c_str(),
                      (long long)blk.ntimes, FJSPH_MAX_TIMES);
                return false;
            }
            L.n_times = (int32_t)blk.ntimes;
            for (size_t t = 0; t < blk.times.size() && t < FJSPH_MAX_TIMES; ++t) L.times[t] = blk.times[t];
            for (size_t t = 0; t < vels.size(); ++t)
                for (int k = 0; k < 3; ++k) L.vels[t][k] = vels[t][k];
        } else {
            L.n_times = 0;
            for (int k = 0; k < 3; ++k) L.vels[0][k] = v0[k];
        }
        return true;
    };
    for (size_t k = 0; k < g.bound.size(); ++k) {
        const Block &blk = g.bound[k];
        fjsph_block L = base_limits(blk, false);
        for (size_t i = 0; i < blk.coords.size(); ++i)
            if (!blk.intersect[i]) push(blk.coords[i], blk, s.bnd_mass, FJSPH_BOUND);
        std::vector<V> vels = blk.vels;
        if (!blk.times.empty()) {
            if (!blk.pos.empty() && blk.vels.empty()) { /* get_boundary_velocity, Init.cpp:27-39 */
                vels.clear();
                for (size_t t = 0; t + 1 < (size_t)blk.ntimes; ++t)
                    vels.push_back(vdiv(vsub(blk.pos[t + 1], blk.pos[t]), blk.times[t + 1] - blk.times[t]));
            } else if (blk.vels.empty()) {
                g.msg("boundary block %zu has motion times but no positions or velocities for them", k);
                return FJSPH_E_ARG;
            }
        }
        if (!set_times(L, blk, vels, blk.vel)) return FJSPH_E_UNSUPPORTED;
        L.second = id;
        g.limits.push_back(L);
    }
    g.n_bound_points = id;
    for (size_t k = 0; k < g.fluid.size(); ++k) {
        const Block &blk = g.fluid[k];
        fjsph_block L = base_limits(blk, true);
        if (blk.bound_type == inletZone) {
            if (blk.particle_order) {
                /* Init_Particles takes five buffer layers for HCP inlets, the generator makes four */
                g.msg("inlet \"%s\" with HCP ordering: the reference reads a fifth buffer layer that its "
                      "inlet generator does not make.", blk.name.c_str());
                return FJSPH_E_UNSUPPORTED;
            }
            const size_t nBuff = 4;
            size_t ii = 0;
            while (ii < blk.bc.size() && blk.bc[ii] == FJSPH_PIPE) {
                /* pipe particles take the boundary mass upstream */
                if (!blk.intersect[ii]) push(blk.coords[ii], blk, s.bnd_mass, FJSPH_PIPE);
                ii++;
            }
            Geometry::Inlet inl;
            inl.block = (int32_t)(g.bound.size() + k);
            std::vector<char> skip(blk.back.size(), 0);
            for (size_t q = 0; q < blk.back.size(); ++q) skip[q] = blk.intersect[(size_t)blk.back[q]] ? 1 : 0;
            for (size_t q = 0; q < blk.back.size(); ++q)
                if (!skip[q]) {
                    inl.back.push_back(id);
                    inl.buffer.emplace_back(nBuff, 0);
                    push(blk.coords[(size_t)blk.back[q]], blk, s.sim_mass, FJSPH_BACK);
                }
            for (size_t layer = 0; layer < nBuff; ++layer) {
                size_t col = 0;
                for (size_t q = 0; q < blk.back.size(); ++q)
                    if (!skip[q]) {
                        inl.buffer[col++][layer] = id;
                        push(blk.coords[(size_t)blk.buffer[q][layer]], blk, s.sim_mass, FJSPH_BUFFER);
                    }
            }
            g.inlets.push_back(std::move(inl));
        } else {
            for (size_t i = 0; i < blk.coords.size(); ++i)
                if (!blk.intersect[i]) push(blk.coords[i], blk, s.sim_mass, FJSPH_FREE);
        }
        L.second = id;
        if (!set_times(L, blk, blk.vels, V{0, 0, 0})) return FJSPH_E_UNSUPPORTED;
        for (int c = 0; c < 3; ++c) {
            L.insert_norm[c] = blk.insert_norm[c];
            L.delete_norm[c] = blk.delete_norm[c];
            L.aero_norm[c] = blk.aero_norm[c];
        }
        if (g.D == 2) L.insert_norm[2] = L.delete_norm[2] = L.aero_norm[2] = 0.0;
        L.insconst = blk.insconst;
        L.delconst = blk.delconst;
        L.aeroconst = blk.aeroconst;
        g.limits.push_back(L);
    }
    if (s.init_hydro_pressure) {
        for (size_t i = 0; i < g.xi.size(); ++i) {
            const double press = std::max(0.0, -s.rho_rest * s.grav[1] * (s.hydro_height - g.xi[i][1]));
            g.p[i] = press;
            g.rho[i] = eos_density(s, press);
        }
    }
    return FJSPH_OK;
}

int build(Geometry &g) {
    int fault = 0;
    g.gs_running = g.s.dx;
    for (auto *set : {&g.bound, &g.fluid})
        for (Block &b : *set) {
            int f = 0;
            check_input(g, b, f);
            if (f) g.msg("block \"%s\" failed its input check", b.name.c_str());
            fault |= f;
        }
    if (fault) {
        g.msg("block input check failed");
        return FJSPH_E_ARG;
    }
    for (auto *set : {&g.bound, &g.fluid})
        for (Block &b : *set) {
            b.coords.reserve((size_t)std::max<int64_t>(b.npts, 1));
            generate(g, b);
            b.generated = (int64_t)b.coords.size();
            if (b.generated != b.npts)
                g.msg("block \"%s\": generated point count is off from the expected count by %d",
                      b.name.c_str(), (int)(b.npts - b.generated));
            b.npts = b.generated;
        }
    check_intersection(g);
    return assemble(g);
}

} // namespace

struct fjsph_geometry {
    Geometry g;
    int pending_fault = 0;
    size_t bound_read = 0, fluid_read = 0; /* blocks read per file, to run check_input once */
};

extern "C" {

int fjsph_geometry_create(const fjsph_settings *s, fjsph_geometry **out) {
    if (!s || !out || (s->dim != 2 && s->dim != 3) || !(s->dx > 0)) return FJSPH_E_ARG;
    auto *h = new fjsph_geometry();
    h->g.s = *s;
    h->g.D = s->dim;
    *out = h;
    return FJSPH_OK;
}

int fjsph_geometry_destroy(fjsph_geometry *h) {
    delete h;
    return FJSPH_OK;
}

int fjsph_geometry_read(fjsph_geometry *h, const char *text, int32_t fluid) {
    if (!h || !text || h->g.built) return FJSPH_E_ARG;
    const int f = read_bmap(h->g, std::string(text), fluid ? h->g.fluid : h->g.bound);
    h->pending_fault |= f;
    return f ? FJSPH_E_ARG : FJSPH_OK;
}

int fjsph_geometry_read_file(fjsph_geometry *h, const char *path, int32_t fluid) {
    if (!h || !path) return FJSPH_E_ARG;
    std::ifstream in(path, std::ios::in | std::ios::binary);
    if (!in.is_open()) {
        h->g.msg("cannot open block file %s", path);
        return FJSPH_E_ARG;
    }
    std::stringstream ss;
    ss << in.rdbuf();
    return fjsph_geometry_read(h, ss.str().c_str(), fluid);
}

int fjsph_geometry_build(fjsph_geometry *h) {
    if (!h || h->g.built) return FJSPH_E_ARG;
    if (h->pending_fault) return FJSPH_E_ARG;
    const int rc = build(h->g);
    if (rc == FJSPH_OK) h->g.built = true;
    return rc;
}

int fjsph_geometry_sizes(const fjsph_geometry *h, int64_t *n_points, int64_t *n_bound_points,
                         int32_t *n_bound_blocks, int32_t *n_fluid_blocks, int32_t *n_inlets) {
    if (!h || !h->g.built) return FJSPH_E_STATE;
    if (n_points) *n_points = (int64_t)h->g.xi.size();
    if (n_bound_points) *n_bound_points = h->g.n_bound_points;
    if (n_bound_blocks) *n_bound_blocks = (int32_t)h->g.bound.size();
    if (n_fluid_blocks) *n_fluid_blocks = (int32_t)h->g.fluid.size();
    if (n_inlets) *n_inlets = (int32_t)h->g.inlets.size();
    return FJSPH_OK;
}

int fjsph_geometry_state(const fjsph_geometry *h, fjsph_state_view *out) {
    if (!h || !out) return FJSPH_E_ARG;
    if (!h->g.built) return FJSPH_E_STATE;
    const Geometry &g = h->g;
    const int D = g.D;
    const int64_t n = (int64_t)g.xi.size();
    if (out->n < n) return FJSPH_E_CAPACITY;
    auto vec = [&](double *dst, const V &val, int64_t i) {
        if (dst)
            for (int k = 0; k < D; ++k) dst[i * D + k] = val[k];
    };
    auto zero_vec = [&](double *dst) {
        if (dst) std::memset(dst, 0, sizeof(double) * (size_t)(n * D));
    };
    auto zero = [&](double *dst) {
        if (dst) std::memset(dst, 0, sizeof(double) * (size_t)n);
    };
    for (double *p : {out->acc, out->Af, out->aVisc, out->gradRho, out->norm, out->vPert}) zero_vec(p);
    if (out->L) std::memset(out->L, 0, sizeof(double) * (size_t)(n * D * D));
    for (double *p : {out->Rrho, out->curve, out->norm_curve, out->woccl, out->pDist, out->deltaD, out->colourG,
                      out->colour, out->lam, out->lam_nb, out->kernsum})
        zero(p);
    const V vinf{g.s.v_inf[0], g.s.v_inf[1], g.s.v_inf[2]};
    for (int64_t i = 0; i < n; ++i) {
        vec(out->xi, g.xi[(size_t)i], i);
        vec(out->v, g.v[(size_t)i], i);
        /* the constant-velocity air source (src/FJSPH.cpp:116-127) */
        vec(out->cellV, vinf, i);
        if (out->rho) out->rho[i] = g.rho[(size_t)i];
        if (out->p) out->p[i] = g.p[(size_t)i];
        if (out->m) out->m[i] = g.m[(size_t)i];
        if (out->cellP) out->cellP[i] = g.s.p_ref;
        if (out->cellRho) out->cellRho[i] = g.s.rho_g;
        if (out->part_id) out->part_id[i] = i;
        if (out->cellID) out->cellID[i] = -3; /* c_no_cell */
        if (out->b) out->b[i] = g.b[(size_t)i];
        if (out->surf) out->surf[i] = 0;
        if (out->surfzone) out->surfzone[i] = 0;
    }
    return FJSPH_OK;
}

int fjsph_geometry_blocks(const fjsph_geometry *h, fjsph_block *blocks, int32_t max_blocks) {
    if (!h || !blocks) return FJSPH_E_ARG;
    if (!h->g.built) return FJSPH_E_STATE;
    if ((size_t)max_blocks < h->g.limits.size()) return FJSPH_E_CAPACITY;
    for (size_t k = 0; k < h->g.limits.size(); ++k) blocks[k] = h->g.limits[k];
    return FJSPH_OK;
}

int fjsph_geometry_block_info(const fjsph_geometry *h, int32_t k, fjsph_geometry_block *info) {
    if (!h || !info) return FJSPH_E_ARG;
    const Geometry &g = h->g;
    const size_t nb = g.bound.size(), nall = nb + g.fluid.size();
    if (k < 0 || (size_t)k >= nall) return FJSPH_E_ARG;
    const Block &b = (size_t)k < nb ? g.bound[(size_t)k] : g.fluid[(size_t)k - nb];
    std::memset(info, 0, sizeof *info);
    std::snprintf(info->name, sizeof info->name, "%s", b.name.c_str());
    info->is_fluid = (size_t)k >= nb ? 1 : 0;
    info->shape = b.bound_type;
    info->sub_shape = b.sub_bound_type;
    info->particle_order = b.particle_order ? 1 : 0;
    info->write_data = b.write_data ? 1 : 0;
    info->ni = b.ni;
    info->nj = b.nj;
    info->nk = b.nk;
    info->estimated = b.estimated;
    info->generated = b.generated;
    info->kept = b.kept;
    info->radius = b.radius;
    for (int c = 0; c < 3; ++c) {
        info->start[c] = b.start[c];
        info->end[c] = b.end[c];
        info->right[c] = b.right[c];
        info->centre[c] = b.centre[c];
        info->normal[c] = b.normal[c];
    }
    return FJSPH_OK;
}

int fjsph_geometry_inlet(const fjsph_geometry *h, int32_t k, fjsph_inlet *inlet) {
    if (!h || !inlet) return FJSPH_E_ARG;
    if (!h->g.built) return FJSPH_E_STATE;
    if (k < 0 || (size_t)k >= h->g.inlets.size()) return FJSPH_E_ARG;
    const Geometry::Inlet &in = h->g.inlets[(size_t)k];
    const int64_t nback = (int64_t)in.back.size(), depth = 4;
    inlet->block = in.block;
    if (!inlet->back || !inlet->buffer) { /* size query */
        inlet->n_back = nback;
        inlet->depth = depth;
        return FJSPH_OK;
    }
    if (inlet->n_back < nback || inlet->depth < depth) return FJSPH_E_CAPACITY;
    inlet->n_back = nback;
    inlet->depth = depth;
    for (int64_t q = 0; q < nback; ++q) {
        inlet->back[q] = in.back[(size_t)q];
        for (int64_t l = 0; l < depth; ++l) inlet->buffer[q * depth + l] = in.buffer[(size_t)q][(size_t)l];
    }
    return FJSPH_OK;
}

int fjsph_geometry_log(const fjsph_geometry *h, char *buf, int64_t cap, int64_t *len) {
    if (!h) return FJSPH_E_ARG;
    const std::string &log = h->g.log;
    if (len) *len = (int64_t)log.size();
    if (buf && cap > 0) {
        const size_t n = std::min((size_t)(cap - 1), log.size());
        std::memcpy(buf, log.data(), n);
        buf[n] = '\0';
    }
    return FJSPH_OK;
}

} // extern "C"
