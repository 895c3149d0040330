// factory/ObjectFactory.h -- stand-in for the reference's plugin factory
// base, used only when the reference's hot-path sources are compiled for the
// parity pins.  The pins construct reference objects directly from
// Parameters, so no factory ever runs; this keeps the declarations the
// sources name.
#pragma once
#include "core/Parameters.h"

#include <memory>
#include <stdexcept>
#include <string>

template <class T>
struct ObjectStaticType {
    static const char *get() { return "unregistered"; }
};

template <class BaseType>
class ObjectFactory {
public:
    typedef std::shared_ptr<ObjectFactory> ptr;
    explicit ObjectFactory(const std::string &type) : myType(type) {}
    virtual ~ObjectFactory() {}
    const std::string &getObjectType() const { return myType; }
    virtual typename BaseType::ptr create(const Parameters &params) = 0;

protected:
    std::string myType;
};

template <class BaseType, class ObjectType, typename... Args>
class TplObjectFactory : public ObjectFactory<BaseType> {
public:
    TplObjectFactory() : ObjectFactory<BaseType>(ObjectStaticType<ObjectType>::get()) {}
    typename BaseType::ptr create(const Parameters &params) override
    {
        return typename BaseType::ptr(new ObjectType(params));
    }
};
