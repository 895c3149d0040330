// factory/ObjectFactoryManager.h -- stand-in for the reference's plugin
// registry in the parity-pin build.  The registration macros expand to
// nothing (no static registrars run); a lookup reports that the registry is
// absent.  Only the scene-file loader looks factories up, and the pin build
// does not compile it.
#pragma once
#include "factory/ObjectFactory.h"

#include <map>
#include <stdexcept>
#include <string>

template <class ReturnType>
class ObjectFactoryManager {
public:
    static ObjectFactoryManager *getInstance()
    {
        static ObjectFactoryManager m;
        return &m;
    }
    void addFactory(typename ObjectFactory<ReturnType>::ptr) {}
    void removeFactory(const std::string &) {}
    typename ObjectFactory<ReturnType>::ptr getFactory(const std::string &type)
    {
        throw std::runtime_error("no plugin registry in the parity-pin build: " + type);
    }
    std::string formatType(const std::string &s) { return s; }
};

#define RT_REGISTER_TYPE(ObjectType, BaseType)
#define RT_REGISTER_TYPE_WITH_FACTORY(ObjectType, BaseType, Factory)
