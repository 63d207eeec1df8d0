// Drives kvs::cuda::MarchingCubes the way user code drives kvs::MarchingCubes
// (Example/Visualization/Isosurface/main.cpp:36-44): a Hydrogen volume, iso =
// (min+max)/2, the constructor form and the pipeline-module form.  Prints one
// line per call: success flag, vertex count, connection count, colour.
#include <cstdio>
#include <kvs/HydrogenVolumeData>
#include <kvs/TransferFunction>
#include "kvs/cuda/MarchingCubes.h"
#include "kvs/cuda/Isosurface.h"
#include "kvs/cuda/SlicePlane.h"
#include "kvs/cuda/MarchingCells.h"
#include <kvs/UnstructuredVolumeObject>

int main()
{
    kvs::HydrogenVolumeData data( kvs::Vec3u( 32, 32, 32 ) );
    kvs::StructuredVolumeObject* volume = data.exec();
    volume->updateMinMaxValues();
    const double iso = ( volume->minValue() + volume->maxValue() ) * 0.5;
    const kvs::TransferFunction tf( 256 );

    kvs::cuda::MarchingCubes* a = new kvs::cuda::MarchingCubes( volume, iso, kvs::PolygonObject::PolygonNormal, true, tf );
    std::printf( "ctor success=%d vertices=%zu connections=%zu\n", a->isSuccess() ? 1 : 0,
                 a->numberOfVertices(), a->numberOfConnections() );

    kvs::cuda::MarchingCubes m;               // PipelineModule form
    m.setIsolevel( iso );
    m.setNormalType( kvs::PolygonObject::VertexNormal );
    kvs::ObjectBase* r = m.exec( volume );
    std::printf( "exec success=%d returned=%d module=%s\n", m.isSuccess() ? 1 : 0, r ? 1 : 0, m.moduleName() );

    kvs::ObjectBase* none = m.exec( nullptr );
    std::printf( "null success=%d returned=%d\n", m.isSuccess() ? 1 : 0, none ? 1 : 0 );

    // kvs::Isosurface's forms (Isosurface.h:35-48) on the drop-in
    kvs::cuda::Isosurface* s = new kvs::cuda::Isosurface( volume, iso, kvs::PolygonObject::PolygonNormal, true, tf );
    std::printf( "isosurface vertices=%zu connections=%zu module=%s\n", s->numberOfVertices(),
                 s->numberOfConnections(), s->moduleName() );
    kvs::cuda::Isosurface t;
    kvs::ObjectBase* u = t.exec( volume );
    std::printf( "isosurface exec returned=%d vertices=%zu\n", u ? 1 : 0, t.numberOfVertices() );
    std::printf( "isosurface null returned=%d\n", t.exec( nullptr ) ? 1 : 0 );
    // kvs::SlicePlane's forms (SlicePlane.h:39-48) on the drop-in
    kvs::cuda::SlicePlane* sp = new kvs::cuda::SlicePlane( volume, kvs::Vec4( 0, 0, 1, -15.5f ), tf );
    std::printf( "slice vertices=%zu module=%s\n", sp->numberOfVertices(), sp->moduleName() );
    kvs::cuda::SlicePlane sq;
    sq.setPlane( kvs::Vec3( 15.0f, 15.0f, 15.0f ), kvs::Vec3( 0.3f, -0.5f, 0.8f ) );
    std::printf( "slice exec returned=%d\n", sq.exec( volume ) ? 1 : 0 );
    // the unstructured mappers (MarchingTetrahedra.h:23-60 and alike): one tetrahedron
    kvs::UnstructuredVolumeObject* tv = new kvs::UnstructuredVolumeObject();
    const kvs::Real32 tc[12] = { 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1 };
    const kvs::UInt32 tk[4] = { 0, 1, 2, 3 };
    const kvs::Real32 tval[4] = { 0, 1, 0, 0 };
    tv->setCellTypeToTetrahedra();
    tv->setVeclen( 1 );
    tv->setNumberOfNodes( 4 );
    tv->setNumberOfCells( 1 );
    tv->setCoords( kvs::ValueArray<kvs::Real32>( tc, 12 ) );
    tv->setConnections( kvs::ValueArray<kvs::UInt32>( tk, 4 ) );
    tv->setValues( kvs::ValueArray<kvs::Real32>( tval, 4 ) );
    kvs::cuda::MarchingTetrahedra* mt = new kvs::cuda::MarchingTetrahedra( tv, 0.5, kvs::PolygonObject::PolygonNormal, true, tf );
    std::printf( "cells vertices=%zu module=%s\n", mt->numberOfVertices(), mt->moduleName() );
    kvs::cuda::MarchingHexahedra mh;
    mh.setIsolevel( 0.5 );
    std::printf( "cells wrong type returned=%d\n", mh.exec( tv ) ? 1 : 0 );
    kvs::cuda::Isosurface ti( tv, 0.5, kvs::PolygonObject::PolygonNormal, true, tf );
    std::printf( "cells isosurface vertices=%zu\n", ti.numberOfVertices() );
    delete mt;
    delete tv;
    delete sp;
    delete s;
    delete a;
    return 0;
}
