/*****************************************************************************/
/**
 *  @file   SlicePlane.cpp
 *  @brief  kvs::cuda::SlicePlane on libkvsmc.
 *
 *  The flow is the reference's (Source/Core/Visualization/Mapper/SlicePlane.cpp):
 *  exec (:60-80) checks the input; mapping (:88-145) checks veclen, attaches
 *  the volume, sets the colour map range (MapperBase::setRange) and the
 *  bounding box, and extracts.  What changes: the min/max behind the colour
 *  range comes from the device scan (filled into the volume's cache first, so
 *  setRange does no CPU scan), and every cell -- of a structured volume, or of
 *  an unstructured one of tetrahedra, hexahedra, pyramids or prisms -- is
 *  handled by libkvsmc's kernels; the arrays arrive as kvs::ValueArrays from
 *  the C call's allocator.  As in the reference, isSuccess() is never set true
 *  by this mapper (MapperBase starts false).
 */
/*****************************************************************************/
#include "SlicePlane.h"

#include <kvs/Message>
#include <kvs/StructuredVolumeObject>
#include <kvs/UnstructuredVolumeObject>
#include <kvs/ValueArray>

#include <limits>

#include "Context.h"
#include "MarchingCells.h"

namespace
{

struct SliceOutputs
{
    kvs::ValueArray<kvs::Real32> coords;
    kvs::ValueArray<kvs::Real32> normals;
    kvs::ValueArray<kvs::UInt8> colors;
};

void* AllocateSlice( void* user, int32_t which, uint64_t count )
{
    SliceOutputs* o = static_cast<SliceOutputs*>( user );
    switch ( which )
    {
    case 0: o->coords.allocate( count ); return o->coords.data();
    case 1: o->normals.allocate( count ); return o->normals.data();
    case 3: o->colors.allocate( count ); return o->colors.data();
    default: return nullptr;
    }
}

} // end of namespace

namespace kvs
{

namespace cuda
{

SlicePlane::SlicePlane(
    const kvs::VolumeObjectBase* volume,
    const kvs::Vec4& coefficients,
    const kvs::TransferFunction& transfer_function ):
    kvs::MapperBase( transfer_function ),
    kvs::PolygonObject()
{
    this->setPlane( coefficients );
    this->exec( volume );
}

SlicePlane::SlicePlane(
    const kvs::VolumeObjectBase* volume,
    const kvs::Vec3& point,
    const kvs::Vec3& normal,
    const kvs::TransferFunction& transfer_function ):
    kvs::MapperBase( transfer_function ),
    kvs::PolygonObject()
{
    this->setPlane( point, normal );
    this->exec( volume );
}

SlicePlane::SuperClass* SlicePlane::exec( const kvs::ObjectBase* object )
{
    if ( !object )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input object is NULL.");
        return nullptr;
    }
    const auto* volume = kvs::VolumeObjectBase::DownCast( object );
    if ( !volume )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input object is not volume dat.");
        return nullptr;
    }
    if ( !this->mapping( volume ) ) return nullptr;
    return this;
}

bool SlicePlane::mapping( const kvs::VolumeObjectBase* volume )
{
    if ( volume->veclen() != 1 )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Input volume is not a sclar field data.");
        return true;   // the reference returns `this` here
    }

    if ( volume->volumeType() != kvs::VolumeObjectBase::Structured )
    {
        return this->mapping_cells( kvs::UnstructuredVolumeObject::DownCast( volume ) );
    }

    const auto* svolume = kvs::StructuredVolumeObject::DownCast( volume );
    const int dtype = kvs::cuda::DType( svolume->values() );
    if ( dtype < 0 )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Unsupported data type '%s'.", svolume->values().typeInfo()->typeName() );
        return true;
    }
    kvsmc_status st = KVSMC_OK;
    kvsmc_context* ctx = kvs::cuda::DeviceContext( m_device, &st );
    if ( !ctx )
    {
        kvsMessageError("libkvsmc: %s.", kvsmc_status_string( st ) );
        return false;
    }
    const auto res = svolume->resolution();
    kvsmc_volume* dvol = nullptr;
    st = kvsmc_volume_upload( ctx, svolume->values().data(), kvsmc_dtype( dtype ), res.x(), res.y(), res.z(), &dvol );
    if ( st == KVSMC_OK && !svolume->hasMinMaxValues() )
    {
        double mn = 0, mx = 0;
        st = kvsmc_volume_minmax( ctx, dvol, &mn, &mx );
        if ( st == KVSMC_OK ) svolume->setMinMaxValues( mn, mx );   // the cache is mutable in the reference too
    }
    if ( st != KVSMC_OK )
    {
        if ( dvol ) kvsmc_volume_free( ctx, dvol );
        kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
        return false;
    }

    BaseClass::attachVolume( volume );
    BaseClass::setRange( volume );
    BaseClass::setMinMaxCoords( volume, this );

    kvsmc_slice_params p;
    for ( int k = 0; k < 4; ++k ) p.coefficients[k] = m_coef[k];
    const kvs::Vec3u ncells( res - kvs::Vec3u::Constant( 1 ) );
    const auto min_coord = volume->minObjectCoord();
    const auto max_coord = volume->maxObjectCoord();
    const auto scale_factor = ( max_coord - min_coord ) / kvs::Vec3{ ncells };   // SlicePlane.cpp:155-157
    for ( int k = 0; k < 3; ++k ) { p.min_coord[k] = min_coord[k]; p.scale[k] = scale_factor[k]; }
    const kvs::ColorMap& cmap = BaseClass::transferFunction().colorMap();
    p.tf_min = cmap.minValue();
    p.tf_max = cmap.maxValue();
    p.tf_resolution = static_cast<int32_t>( cmap.resolution() );
    p.tf_table = cmap.table().data();
    SliceOutputs out;
    uint64_t ntriangles = 0;
    st = kvsmc_slice_plane( ctx, dvol, &p, &AllocateSlice, &out, &ntriangles );
    kvsmc_volume_free( ctx, dvol );
    if ( st != KVSMC_OK )
    {
        kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
        return false;
    }
    // SlicePlane.cpp:196-202
    SuperClass::setCoords( out.coords );
    SuperClass::setColors( out.colors );
    SuperClass::setNormals( out.normals );
    SuperClass::setOpacity( 255 );
    SuperClass::setPolygonType( kvs::PolygonObject::Triangle );
    SuperClass::setColorType( kvs::PolygonObject::VertexColor );
    SuperClass::setNormalType( kvs::PolygonObject::PolygonNormal );
    return true;
}

// The unstructured branch (SlicePlane.cpp:128-147, 291-800): the cells of a
// tetrahedral, hexahedral, pyramidal or prismatic volume on the GPU
// (kvsmc_slice_cells_host), the min/max behind the colour range from the
// device scan over the cells' nodes; other cell types give nothing.
bool SlicePlane::mapping_cells( const kvs::UnstructuredVolumeObject* volume )
{
    int cell = -1;
    switch ( volume->cellType() )
    {
    case kvs::UnstructuredVolumeObject::Tetrahedra: cell = KVSMC_TETRAHEDRA; break;
    case kvs::UnstructuredVolumeObject::Hexahedra: cell = KVSMC_HEXAHEDRA; break;
    case kvs::UnstructuredVolumeObject::Pyramid: cell = KVSMC_PYRAMID; break;
    case kvs::UnstructuredVolumeObject::Prism: cell = KVSMC_PRISM; break;
    default: break;
    }
    const int dtype = kvs::cuda::DType( volume->values() );
    kvsmc_status st = KVSMC_OK;
    kvsmc_context* ctx = nullptr;
    if ( cell >= 0 && dtype >= 0 )
    {
        ctx = kvs::cuda::DeviceContext( m_device, &st );
        if ( !ctx )
        {
            kvsMessageError("libkvsmc: %s.", kvsmc_status_string( st ) );
            return false;
        }
        if ( !volume->hasMinMaxValues() )
        {
            // at isolevel NaN no node is above: only the min/max scan runs
            kvsmc_sizes sizes{};
            st = kvsmc_marching_cells_host( ctx, kvsmc_cell_type( cell ), volume->values().data(),
                                            kvsmc_dtype( dtype ), volume->numberOfNodes(), volume->coords().data(),
                                            volume->connections().data(), volume->numberOfCells(),
                                            std::numeric_limits<double>::quiet_NaN(), 0, 0.0, 0.0,
                                            []( void*, int32_t, uint64_t ) -> void* { return nullptr; }, nullptr,
                                            &sizes );
            if ( st != KVSMC_OK )
            {
                kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
                return false;
            }
            volume->setMinMaxValues( sizes.min_value, sizes.max_value );
        }
    }
    BaseClass::attachVolume( volume );
    BaseClass::setRange( volume );
    if ( cell >= 0 && !volume->hasMinMaxObjectCoords() && volume->coords().size() > 0 )
    {
        if ( !kvs::cuda::DeviceBounds( volume, cell, m_device ) ) return false;
    }
    BaseClass::setMinMaxCoords( volume, this );
    if ( dtype < 0 )
    {
        BaseClass::setSuccess( false );
        kvsMessageError("Unsupported data type '%s'.", volume->values().typeInfo()->typeName() );
        return true;
    }
    if ( cell < 0 ) return true;   // extract_plane: default: break

    kvsmc_slice_params p;
    for ( int k = 0; k < 4; ++k ) p.coefficients[k] = m_coef[k];
    for ( int k = 0; k < 3; ++k ) { p.min_coord[k] = 0.0f; p.scale[k] = 1.0f; }
    const kvs::ColorMap& cmap = BaseClass::transferFunction().colorMap();
    p.tf_min = cmap.minValue();
    p.tf_max = cmap.maxValue();
    p.tf_resolution = static_cast<int32_t>( cmap.resolution() );
    p.tf_table = cmap.table().data();
    SliceOutputs out;
    uint64_t ntriangles = 0;
    st = kvsmc_slice_cells_host( ctx, kvsmc_cell_type( cell ), volume->values().data(), kvsmc_dtype( dtype ),
                                 volume->numberOfNodes(), volume->coords().data(), volume->connections().data(),
                                 volume->numberOfCells(), &p, &AllocateSlice, &out, &ntriangles );
    if ( st != KVSMC_OK )
    {
        kvsMessageError("libkvsmc: %s: %s", kvsmc_status_string( st ), kvsmc_last_error( ctx ) );
        return false;
    }
    SuperClass::setCoords( out.coords );
    SuperClass::setColors( out.colors );
    SuperClass::setNormals( out.normals );
    SuperClass::setOpacity( 255 );
    SuperClass::setPolygonType( kvs::PolygonObject::Triangle );
    SuperClass::setColorType( kvs::PolygonObject::VertexColor );
    SuperClass::setNormalType( kvs::PolygonObject::PolygonNormal );
    return true;
}

} // end of namespace cuda

} // end of namespace kvs
