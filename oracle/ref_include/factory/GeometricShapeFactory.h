// factory/GeometricShapeFactory.h -- stand-in for the reference's shape
// factory in the parity-pin build (see factory/ObjectFactoryManager.h): the
// pins build shapes directly, so only the name is kept.
#pragma once
#include "factory/ObjectFactory.h"

template <class BaseType, class ObjectType>
class GeometricShapeFactory;
