// Runs the KVS drop-ins kvs::cuda::MarchingCubes and kvs::cuda::Isosurface
// beside the reference's kvs::MarchingCubes and kvs::Isosurface in one
// process, on twin copies of the same volumes, and compares what they leave
// behind bit for bit: coords, normals, connections, colour, opacity, the
// polygon / normal / colour types, the bounding boxes, the success flag and
// the volume's min/max cache.  Linked against a stand-in of the C ABI whose
// per-cell work is the oracle's (tests/kvs_adapter/oracle_backend.c), so what
// is compared is the drop-ins' host logic: the parameters they hand to the C
// ABI and what they make of its answer.  Prints "cases=N mismatches=M" last.
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include <kvs/HydrogenVolumeData>
#include <kvs/Isosurface>
#include <kvs/MarchingCubes>
#include <kvs/StructuredVolumeObject>
#include <kvs/TransferFunction>

#include "kvs/cuda/Isosurface.h"
#include "kvs/cuda/MarchingCubes.h"

namespace
{

int g_cases = 0;
int g_mismatches = 0;

template <typename A>
bool same_bytes( const A& a, const A& b )
{
    return a.byteSize() == b.byteSize() && ( a.byteSize() == 0 || std::memcmp( a.data(), b.data(), a.byteSize() ) == 0 );
}

bool same_vec( const kvs::Vec3& a, const kvs::Vec3& b ) { return std::memcmp( &a, &b, sizeof a ) == 0; }

bool same_double( double a, double b ) { return std::memcmp( &a, &b, sizeof a ) == 0; }

void check( const char* tag, const kvs::PolygonObject& r, bool r_ok, const kvs::StructuredVolumeObject& rv,
            const kvs::PolygonObject& g, bool g_ok, const kvs::StructuredVolumeObject& gv )
{
    ++g_cases;
    const char* what = nullptr;
    if ( r_ok != g_ok ) what = "success";
    else if ( !same_bytes( r.coords(), g.coords() ) ) what = "coords";
    else if ( !same_bytes( r.normals(), g.normals() ) ) what = "normals";
    else if ( !same_bytes( r.connections(), g.connections() ) ) what = "connections";
    else if ( !same_bytes( r.colors(), g.colors() ) ) what = "colors";
    else if ( !same_bytes( r.opacities(), g.opacities() ) ) what = "opacities";
    else if ( r.polygonType() != g.polygonType() ) what = "polygon type";
    else if ( r.normalType() != g.normalType() ) what = "normal type";
    else if ( r.colorType() != g.colorType() ) what = "color type";
    else if ( !same_vec( r.minObjectCoord(), g.minObjectCoord() ) || !same_vec( r.maxObjectCoord(), g.maxObjectCoord() ) )
        what = "object coords";
    else if ( !same_vec( r.minExternalCoord(), g.minExternalCoord() ) ||
              !same_vec( r.maxExternalCoord(), g.maxExternalCoord() ) )
        what = "external coords";
    else if ( rv.hasMinMaxValues() != gv.hasMinMaxValues() ||
              ( rv.hasMinMaxValues() &&
                ( !same_double( rv.minValue(), gv.minValue() ) || !same_double( rv.maxValue(), gv.maxValue() ) ) ) )
        what = "volume min/max";
    if ( what )
    {
        ++g_mismatches;
        std::printf( "MISMATCH %s: %s (vertices %zu vs %zu)\n", tag, what, r.numberOfVertices(), g.numberOfVertices() );
    }
}

template <typename T>
kvs::StructuredVolumeObject* make_volume( const std::vector<T>& v, unsigned nx, unsigned ny, unsigned nz )
{
    auto* vol = new kvs::StructuredVolumeObject();
    vol->setGridTypeToUniform();
    vol->setVeclen( 1 );
    vol->setResolution( kvs::Vec3u( nx, ny, nz ) );
    vol->setValues( kvs::ValueArray<T>( v.data(), v.size() ) );
    return vol;
}

struct Mode
{
    kvs::PolygonObject::NormalType nt;
    bool dup;
};
const Mode kModes[] = { { kvs::PolygonObject::PolygonNormal, true },
                        { kvs::PolygonObject::PolygonNormal, false },
                        { kvs::PolygonObject::VertexNormal, true } };

// One volume (made twice by `make`), the mapper in its constructor form and
// in the pipeline form, and kvs::Isosurface's three forms.
template <typename Make>
void run_volume( const char* name, Make make, const std::vector<double>& isos, bool preset_minmax )
{
    const kvs::TransferFunction tf( 256 );
    char tag[256];
    for ( double iso : isos )
    {
        for ( const Mode& m : kModes )
        {
            std::snprintf( tag, sizeof tag, "%s iso=%g nt=%d dup=%d mc", name, iso, (int)m.nt, (int)m.dup );
            kvs::StructuredVolumeObject* rv = make();
            kvs::StructuredVolumeObject* gv = make();
            if ( preset_minmax )
            {
                rv->setMinMaxValues( 0.25, 0.75 );
                gv->setMinMaxValues( 0.25, 0.75 );
            }
            kvs::MarchingCubes r( rv, iso, m.nt, m.dup, tf );
            kvs::cuda::MarchingCubes g( gv, iso, m.nt, m.dup, tf );
            check( tag, r, r.isSuccess(), *rv, g, g.isSuccess(), *gv );

            std::snprintf( tag, sizeof tag, "%s iso=%g nt=%d dup=%d pipeline", name, iso, (int)m.nt, (int)m.dup );
            kvs::MarchingCubes rp;
            kvs::cuda::MarchingCubes gp;
            rp.setIsolevel( iso );
            gp.setIsolevel( iso );
            rp.setNormalType( m.nt );
            gp.setNormalType( m.nt );
            const bool r_ok = rp.exec( rv ) != nullptr;
            const bool g_ok = gp.exec( gv ) != nullptr;
            check( tag, rp, r_ok, *rv, gp, g_ok, *gv );

            std::snprintf( tag, sizeof tag, "%s iso=%g nt=%d dup=%d isosurface", name, iso, (int)m.nt, (int)m.dup );
            kvs::Isosurface ri( rv, iso, m.nt, m.dup, tf );
            kvs::cuda::Isosurface gi( gv, iso, m.nt, m.dup, tf );
            check( tag, ri, ri.isSuccess(), *rv, gi, gi.isSuccess(), *gv );
            delete rv;
            delete gv;
        }
    }
    for ( const Mode& m : kModes )
    {
        // kvs::Isosurface( volume, normal_type ): isolevel (max + min) / 2 from the
        // volume's min/max cache, filled first (Isosurface.cpp:23-40)
        std::snprintf( tag, sizeof tag, "%s nt=%d isosurface default isolevel", name, (int)m.nt );
        kvs::StructuredVolumeObject* rv = make();
        kvs::StructuredVolumeObject* gv = make();
        kvs::Isosurface ri( rv, m.nt );
        kvs::cuda::Isosurface gi( gv, m.nt );
        check( tag, ri, ri.isSuccess(), *rv, gi, gi.isSuccess(), *gv );
        std::snprintf( tag, sizeof tag, "%s nt=%d isosurface (volume, iso, nt)", name, (int)m.nt );
        kvs::Isosurface rj( rv, isos[0], m.nt );
        kvs::cuda::Isosurface gj( gv, isos[0], m.nt );
        check( tag, rj, rj.isSuccess(), *rv, gj, gj.isSuccess(), *gv );
        delete rv;
        delete gv;
    }
}

} // end of namespace

int main()
{
    std::mt19937 rng( 12345 );
    {
        // the reference example's volume (uint8), its values copied out once
        kvs::HydrogenVolumeData data( kvs::Vec3u( 32, 32, 32 ) );
        const kvs::StructuredVolumeObject* h = data.exec();
        if ( h->values().typeID() != kvs::Type::TypeUInt8 ) { std::printf( "hydrogen is not uint8\n" ); return 1; }
        const auto* p = static_cast<const kvs::UInt8*>( h->values().data() );
        std::vector<kvs::UInt8> v( p, p + 32 * 32 * 32 );
        auto make = [&] { return make_volume( v, 32, 32, 32 ); };
        run_volume( "hydrogen32", make, { 127.5, 40.0, 200.0 }, false );
    }
    {
        std::uniform_real_distribution<float> u( 0.0f, 1.0f );
        std::vector<float> v( 17 * 13 * 11 );
        for ( auto& x : v ) x = u( rng );
        auto make = [&] { return make_volume( v, 17, 13, 11 ); };
        run_volume( "random_f32", make, { 0.5, 0.3 }, false );
        run_volume( "random_f32_preset", make, { 0.5 }, true );
    }
    {
        std::uniform_int_distribution<int> u( -300, 300 );
        std::vector<kvs::Int16> v( 9 * 10 * 12 );
        for ( auto& x : v ) x = (kvs::Int16)u( rng );
        auto make = [&] { return make_volume( v, 9, 10, 12 ); };
        run_volume( "random_i16", make, { 0.5, -100.25 }, false );
    }
    {
        std::uniform_int_distribution<int> u( 0, 255 );
        std::vector<kvs::UInt8> v( 8 * 9 * 7 );
        for ( auto& x : v ) x = (kvs::UInt8)u( rng );
        auto make = [&] { return make_volume( v, 8, 9, 7 ); };
        run_volume( "random_u8", make, { 128.0, 31.5 }, false );
    }
    {
        std::uniform_real_distribution<double> u( -1.0, 1.0 );
        std::vector<kvs::Real64> v( 7 * 6 * 9 );
        for ( auto& x : v ) x = u( rng );
        auto make = [&] { return make_volume( v, 7, 6, 9 ); };
        run_volume( "random_f64", make, { 0.0, 0.6 }, false );
    }
    {
        std::vector<float> v( 5 * 5 * 5, 0.5f );   // Math::Equal(min, max): nothing extracted
        auto make = [&] { return make_volume( v, 5, 5, 5 ); };
        run_volume( "constant_f32", make, { 0.5 }, false );
    }
    std::printf( "cases=%d mismatches=%d\n", g_cases, g_mismatches );
    return g_mismatches == 0 ? 0 : 1;
}
