/*****************************************************************************/
/**
 *  @file   MarchingCells.cpp
 *  @brief  kvs::cuda::MarchingTetrahedra / Hexahedra / Pyramid / Prism on
 *          libkvsmc.
 *
 *  The flow is the reference's (Source/Core/Visualization/Mapper/
 *  MarchingTetrahedra.cpp:46-136, MarchingHexahedra.cpp:46-127 and the same
 *  lines of MarchingPyramid.cpp and MarchingPrism.cpp): exec's checks and
 *  messages, VertexNormal forcing duplication off, then mapping -- setRange
 *  (the volume's min/max cache filled by the device scan over the cells'
 *  nodes), setMinMaxCoords, the polygon types, the Math::Equal(min, max)
 *  early exit, the value-type switch, and the duplicated-vertex extraction,
 *  here one kvsmc_marching_cells_host call.
 */
/*****************************************************************************/
#include "MarchingCells.h"

#include <kvs/Math>
#include <kvs/Message>
#include <kvs/ValueArray>

#include <limits>

#include "Context.h"

namespace
{

struct CellOutputs
{
    kvs::ValueArray<kvs::Real32> coords;
    kvs::ValueArray<kvs::Real32> normals;
};

void* AllocateCells( void* user, int32_t which, uint64_t count )
{
    CellOutputs* o = static_cast<CellOutputs*>( user );
    switch ( which )
    {
    case 0: o->coords.allocate( count ); return o->coords.data();
    case 1: o->normals.allocate( count ); return o->normals.data();
    default: return nullptr;
    }
}


} // end of namespace

namespace kvs
{

namespace cuda
{

bool DeviceBounds( const kvs::UnstructuredVolumeObject* volume, int cell, int device )
{
    kvsmc_status st = KVSMC_OK;
    kvsmc_context* ctx = DeviceContext( device, &st );
    if ( !ctx )
    {
        kvsMessageError("libkvsmc: %s.", kvsmc_status_string( st ) );
        return false;
    }
    float lo[3], hi[3];
    st = kvsmc_cells_bounds( ctx, kvsmc_cell_type( cell ), volume->coords().data(), volume->numberOfNodes(),
                             volume->connections().data(), volume->numberOfCells(), lo, hi );
    if ( st != KVSMC_OK )
    {
        kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
        return false;
    }
    // the cache is mutable in the reference too (MapperBase.cpp:101)
    auto* v = const_cast<kvs::UnstructuredVolumeObject*>( volume );
    v->setMinMaxObjectCoords( kvs::Vec3( lo[0], lo[1], lo[2] ), kvs::Vec3( hi[0], hi[1], hi[2] ) );
    if ( !v->hasMinMaxExternalCoords() )
    {
        v->setMinMaxExternalCoords( kvs::Vec3( lo[0], lo[1], lo[2] ), kvs::Vec3( hi[0], hi[1], hi[2] ) );
    }
    return true;
}

} // end of namespace cuda

} // end of namespace kvs

namespace kvs
{

namespace cuda
{

MarchingCellsBase::MarchingCellsBase(
    const kvs::TransferFunction& transfer_function,
    const double isolevel,
    const bool duplication ):
    kvs::MapperBase( transfer_function ),
    m_isolevel( isolevel ),
    m_duplication( duplication )
{
}

MarchingCellsBase::SuperClass* MarchingCellsBase::run( const kvs::ObjectBase* object, const Traits& traits )
{
    if ( !object )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input object is NULL.");
        return nullptr;
    }
    const auto* volume = kvs::UnstructuredVolumeObject::DownCast( object );
    if ( !volume )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input object is not unstructured volume object.");
        return nullptr;
    }
    if ( volume->veclen() != 1 )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input volume is not sclar field data.");
        return nullptr;
    }
    if ( volume->cellType() != traits.type )
    {
        BaseClass::setSuccess( false );
        kvsMessageError( "%s", traits.type_message );
        return nullptr;
    }
    if ( SuperClass::normalType() == kvs::PolygonObject::VertexNormal ) { m_duplication = false; }
    if ( !this->mapping( volume, traits ) ) { return nullptr; }
    return this;
}

bool MarchingCellsBase::mapping( const kvs::UnstructuredVolumeObject* volume, const Traits& traits )
{
    BaseClass::attachVolume( volume );
    const int dtype = DType( volume->values() );
    CellOutputs out;
    kvsmc_sizes sizes{};
    if ( dtype >= 0 && ( m_duplication || !volume->hasMinMaxValues() ) )
    {
        kvsmc_status st = KVSMC_OK;
        kvsmc_context* ctx = DeviceContext( m_device, &st );
        if ( !ctx )
        {
            kvsMessageError("libkvsmc: %s.", kvsmc_status_string( st ) );
            return false;
        }
        // without extraction only the min/max is wanted: at isolevel NaN no
        // node is above, so only the scan and an empty count pass run
        const double iso = m_duplication ? m_isolevel : std::numeric_limits<double>::quiet_NaN();
        st = kvsmc_marching_cells_host(
            ctx, kvsmc_cell_type( traits.cell ), volume->values().data(), kvsmc_dtype( dtype ),
            volume->numberOfNodes(), volume->coords().data(), volume->connections().data(), volume->numberOfCells(),
            iso, volume->hasMinMaxValues() ? 1 : 0, volume->minValue(), volume->maxValue(), &AllocateCells, &out,
            &sizes );
        if ( st != KVSMC_OK )
        {
            kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
            return false;
        }
        if ( !volume->hasMinMaxValues() ) volume->setMinMaxValues( sizes.min_value, sizes.max_value );
    }
    BaseClass::setRange( volume );
    if ( !volume->hasMinMaxObjectCoords() && volume->coords().size() > 0 )
    {
        // UnstructuredVolumeObject::updateMinMaxCoords' fold on the GPU
        if ( !DeviceBounds( volume, traits.cell, m_device ) ) return false;
    }
    BaseClass::setMinMaxCoords( volume, this );

    if ( m_duplication || !traits.types_need_duplication )
    {
        SuperClass::setPolygonType( kvs::PolygonObject::Triangle );
        SuperClass::setColorType( kvs::PolygonObject::PolygonColor );
        SuperClass::setNormalType( kvs::PolygonObject::PolygonNormal );
    }
    if ( kvs::Math::Equal( volume->minValue(), volume->maxValue() ) ) { return true; }
    if ( dtype < 0 )
    {
        BaseClass::setSuccess( false );
        kvsMessageError( traits.dtype_message, volume->values().typeInfo()->typeName() );
        return true;
    }
    if ( m_duplication && out.coords.size() > 0 )
    {
        SuperClass::setCoords( out.coords );
        SuperClass::setColor( BaseClass::transferFunction().colorMap().at( m_isolevel ) );
        SuperClass::setNormals( out.normals );
        SuperClass::setOpacity( 255 );
    }
    return true;
}

#define KVSMC_CELL_MAPPER_DEFS( NAME, CELL, TYPE, TYPE_MESSAGE, DTYPE_MESSAGE, TYPES_NEED_DUP )               \
    NAME::NAME( const kvs::UnstructuredVolumeObject* volume, const double isolevel,                             \
                const SuperClass::NormalType normal_type, const bool duplication,                               \
                const kvs::TransferFunction& transfer_function ):                                               \
        MarchingCellsBase( transfer_function, isolevel, duplication )                                           \
    {                                                                                                           \
        SuperClass::setNormalType( normal_type );                                                               \
        this->exec( volume );                                                                                   \
    }                                                                                                           \
    NAME::SuperClass* NAME::exec( const kvs::ObjectBase* object )                                               \
    {                                                                                                           \
        static const Traits traits = { CELL, kvs::UnstructuredVolumeObject::TYPE, TYPE_MESSAGE, DTYPE_MESSAGE,  \
                                       TYPES_NEED_DUP };                                                        \
        return this->run( object, traits );                                                                     \
    }

KVSMC_CELL_MAPPER_DEFS( MarchingTetrahedra, KVSMC_TETRAHEDRA, Tetrahedra, "Input volume is not tetrahedra-cell data.",
                        "Unsupported data type '%s'.", true )
KVSMC_CELL_MAPPER_DEFS( MarchingHexahedra, KVSMC_HEXAHEDRA, Hexahedra, "Input volume is not hexhedra-cell data.",
                        "Unsupported data type '%s' of the volume.", false )
KVSMC_CELL_MAPPER_DEFS( MarchingPyramid, KVSMC_PYRAMID, Pyramid, "Input volume is not pyramid-cell data.",
                        "Unsupported data type '%s' of the volume.", false )
KVSMC_CELL_MAPPER_DEFS( MarchingPrism, KVSMC_PRISM, Prism, "Input volume is not prism-cell data.",
                        "Unsupported data type '%s' of the volume.", false )

#undef KVSMC_CELL_MAPPER_DEFS

} // end of namespace cuda

} // end of namespace kvs
